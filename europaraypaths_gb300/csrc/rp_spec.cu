// rp_spec.cu -- the fast form's pair kernels beside the default mode's:
// k_pairs32s for specular mode (specular with linear convolution, ttype-1
// targets) and k_pairs32t0 for ttype-0 targets (genRefrPhasor, either mode).
// k_pairs32s: compTargetRays,
// compRefrEnergyIn/Out with their facetReradiation factors, accumulateTarget
// and radiateTarget (geometry_kernels.cu:272-350, 520-584, radar_kernels.cu:
// 767-892).  The two refraction legs carry different reradiation factors, so
// unlike the default mode the outbound leg is binned into its own trace.  Its
// own translation unit (see rp_pair.cuh).
#include <algorithm>

#include "rp_internal.h"
#include "rp_pair.cuh"

namespace rpk {

// Persistent over (trace, target block, part) items, like k_pairs32, with
// the general-frame evaluation (the specular terms need the facet normal).
template <int NT, int ILP, int MINB>
__global__ void __launch_bounds__(RP_PAIR_THREADS, MINB)
k_pairs32s(const __grid_constant__ PairArgs A) {
    RP_PAIR_SMEM_DECL
    const unsigned int items = (unsigned)A.nb * A.tblocks * RP_PARTS;
    for (;;) {
        if (tid == 0) s_item = atomicAdd(A.work, 1u);
        __syncthreads();
        const unsigned int item = s_item;
        __syncthreads();
        if (item >= items) break;
        const int part = item % RP_PARTS;
        const int tb = (item / RP_PARTS) % A.tblocks;
        const int s = item / (RP_PARTS * A.tblocks);
        if (!pair_item<NT, ILP, false, true, RP_WIN>(A, s, tb, part, bars, phase)) break;
    }
    RP_PAIR_SMEM_END
}

// cfg 0: 2 facet pairs per step, 1: 1 (both 2 blocks per SM; the two bin
// windows and staged FacetSpec chunks take 112 KiB of shared memory a block).
template <int NT>
void (*pick_spec_cfg(int cfg))(const PairArgs) {
    return (cfg & 1) ? k_pairs32s<NT, 1, 2> : k_pairs32s<NT, 2, 2>;
}

int launch_pairs_spec(int deg, int cfg, const PairArgs& P, int64_t items, int sms, cudaStream_t st) {
    void (*pk)(const PairArgs);
    switch (deg) {
        case 3: pk = pick_spec_cfg<3>(cfg); break;
        case 4: pk = pick_spec_cfg<4>(cfg); break;
        case 5: pk = pick_spec_cfg<5>(cfg); break;
        case 6: pk = pick_spec_cfg<6>(cfg); break;
        default: pk = pick_spec_cfg<0>(cfg); break;
    }
    const size_t smem = RP_PAIR_SPEC_SMEM_BYTES;
    if (int rc = rp_allow_dyn_smem((const void*)pk, smem)) return rc;
    int occ = 0;
    RP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pk, RP_PAIR_THREADS, smem));
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)std::max(occ, 1) * sms, items));
    pk<<<grid, RP_PAIR_THREADS, smem, st>>>(P);
    return RP_OK;
}

// ttype-0 targets (genRefrPhasor): targets [tq0[s], ntl[s]) of each trace,
// 2 facet pairs per step, 2 blocks per SM.
template <int NT, bool ORTHO, bool SPEC>
__global__ void __launch_bounds__(RP_PAIR_THREADS, 2)
k_pairs32t0(const __grid_constant__ PairArgs A) {
    RP_PAIR_SMEM_DECL
    const unsigned int items = (unsigned)A.nb * A.tblocks * RP_PARTS;
    for (;;) {
        if (tid == 0) s_item = atomicAdd(A.work, 1u);
        __syncthreads();
        const unsigned int item = s_item;
        __syncthreads();
        if (item >= items) break;
        const int part = item % RP_PARTS;
        const int tb = (item / RP_PARTS) % A.tblocks;
        const int s = item / (RP_PARTS * A.tblocks);
        if (!pair_item_t0<NT, 2, ORTHO, SPEC, RP_WIN_WIDE>(A, s, tb, part, bars, phase)) break;
    }
    RP_PAIR_SMEM_END
}

int launch_pairs_t0(int deg, bool ortho, bool spec, const PairArgs& P, int64_t items, int sms, cudaStream_t st) {
    void (*pk)(const PairArgs);
    if (!spec) {
        pk = ortho ? k_pairs32t0<0, true, false> : k_pairs32t0<0, false, false>;
    } else {
        switch (deg) {       // the reradiation polynomials' degree
            case 3: pk = k_pairs32t0<3, false, true>; break;
            case 4: pk = k_pairs32t0<4, false, true>; break;
            case 5: pk = k_pairs32t0<5, false, true>; break;
            case 6: pk = k_pairs32t0<6, false, true>; break;
            default: pk = k_pairs32t0<0, false, true>; break;
        }
    }
    const size_t smem = pair_t0_smem_bytes(RP_WIN_WIDE, spec);
    if (int rc = rp_allow_dyn_smem((const void*)pk, smem)) return rc;
    int occ = 0;
    RP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pk, RP_PAIR_THREADS, smem));
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)std::max(occ, 1) * sms, items));
    pk<<<grid, RP_PAIR_THREADS, smem, st>>>(P);
    return RP_OK;
}

}  // namespace rpk
