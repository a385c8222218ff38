// sn_sweep_inst.cu -- kernels of one cutoff.  Compiled once per cutoff with
// -DSN_RC=<rc> (1..SN_MAX_CUTOFF) so the builds run in parallel and each
// object holds one fully unrolled stencil.  -DSN_PART=1|2|3 compiles only the
// sweep kernels, the FP32-field pass or the FP64 pass of that cutoff (three
// objects that compile in parallel); without it, all of them.
#include "sn_launch.h"
#include "sn_sweep.cuh"

#ifndef SN_RC
#error "compile with -DSN_RC=<cutoff>"
#endif
#ifndef SN_PART
#define SN_PART 0
#endif

#define SN_CAT2(a, b) a##b
#define SN_CAT(a, b) SN_CAT2(a, b)

static_assert(sizeof(SnFieldArgsHost) >= sizeof(sn_sweep::SnFieldArgs), "field args layout");

#if SN_PART == 0 || SN_PART == 1
cudaError_t SN_CAT(sn_launch_sweep_rc, SN_RC)(bool two_d, bool mixed, bool cached, const SnPhaseArgs &a, int grid,
                                              int threads, int smem, cudaStream_t st)
{
    return sn_sweep::launch_rc<SN_RC>(two_d, mixed, cached, a, grid, threads, smem, st);
}

cudaError_t SN_CAT(sn_launch_flow_rc, SN_RC)(bool two_d, bool mixed, bool cached, const SnFlowArgs &a, int grid,
                                             int threads, int smem, cudaStream_t st, int *max_grid)
{
    return sn_sweep::launch_flow_rc<SN_RC>(two_d, mixed, cached, a, grid, threads, smem, st, max_grid);
}

int SN_CAT(sn_cached_smem_rc, SN_RC)(int cslots, int tg, int pc, bool mixed, int ng)
{
    return (int)sn_sweep::sn_ccarve(cslots, tg, pc, sn_sweep::Geo<SN_RC, false>::NP, mixed, ng).total;
}

void SN_CAT(sn_geo_rc, SN_RC)(bool two_d, int *S, int *SZ, int *NS, int *NF, int *merge)
{
    sn_sweep::geo_sizes<SN_RC>(two_d, *S, *SZ, *NS, *NF, *merge);
}
#endif

#if SN_PART == 0 || SN_PART == 3
cudaError_t SN_CAT(sn_launch_field64_rc, SN_RC)(bool two_d, bool mixed, const void *field_args, int grid, int threads,
                                                int smem, cudaStream_t st)
{
    const sn_sweep::SnFieldArgs &fa = *static_cast<const sn_sweep::SnFieldArgs *>(field_args);
    return sn_sweep::launch_field_rc<double, SN_RC>(two_d, mixed, fa, grid, threads, smem, st);
}
#endif

#if SN_PART == 0 || SN_PART == 2
cudaError_t SN_CAT(sn_launch_gfield_rc, SN_RC)(bool mixed, const void *field_args, int grid, int smem,
                                               cudaStream_t st)
{
    const sn_sweep::SnFieldArgs &fa = *static_cast<const sn_sweep::SnFieldArgs *>(field_args);
    return sn_sweep::launch_gfield_rc<SN_RC>(mixed, fa, grid, smem, st);
}

cudaError_t SN_CAT(sn_launch_field_rc, SN_RC)(bool fp64, bool two_d, bool mixed, const void *field_args, int grid,
                                              int threads, int smem, cudaStream_t st)
{
    if (fp64) return SN_CAT(sn_launch_field64_rc, SN_RC)(two_d, mixed, field_args, grid, threads, smem, st);
    const sn_sweep::SnFieldArgs &fa = *static_cast<const sn_sweep::SnFieldArgs *>(field_args);
    return sn_sweep::launch_field_rc<float, SN_RC>(two_d, mixed, fa, grid, threads, smem, st);
}
#endif
