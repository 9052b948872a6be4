// rp_multi.cu -- the multi-job pair kernel: one persistent launch over the
// work items of many batches (scenes of different sizes, bands, bin counts
// and sinc degrees).  Its own translation unit (see rp_pair.cuh).
#include <algorithm>
#include <vector>

#include "rp_internal.h"
#include "rp_pair.cuh"

namespace rpk {

// Multi-job pair kernel: one persistent launch over the items of many
// batches (scenes of different sizes, bin counts and sinc degrees).  Job j
// owns items [start[j], start[j + 1]); a block copies the job's constants
// into registers and dispatches on its sinc degree and facet-frame kind.
template <int ILP, int MINB>
__global__ void __launch_bounds__(RP_PAIR_THREADS, MINB)
k_pairs32m(const PairJob* __restrict__ jobs, const unsigned int* __restrict__ start, int njobs,
           unsigned int* work) {
    RP_PAIR_SMEM_DECL
    __shared__ int s_job;
    const unsigned int total = start[njobs];
    for (;;) {
        if (tid == 0) {
            const unsigned int it = atomicAdd(work, 1u);
            int lo = 0, hi = njobs - 1;          // last j with start[j] <= it
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (start[mid] <= it) lo = mid; else hi = mid - 1;
            }
            s_item = it;
            s_job = lo;
        }
        __syncthreads();
        const unsigned int item = s_item;
        const int j = s_job;
        __syncthreads();
        if (item >= total) break;
        const PairArgs A = jobs[j].a;
        const int deg = jobs[j].deg;
        const int ortho = jobs[j].ortho;
        const unsigned int li = item - start[j];
        const int part = li % RP_PARTS;
        const int tb = (li / RP_PARTS) % A.tblocks;
        const int s = li / (RP_PARTS * A.tblocks);
        bool ok;
        if (ortho) {
            switch (deg) {
                case 3: ok = pair_item<3, ILP, true, false, RP_WIN_WIDE>(A, s, tb, part, bars, phase); break;
                case 4: ok = pair_item<4, ILP, true, false, RP_WIN_WIDE>(A, s, tb, part, bars, phase); break;
                case 5: ok = pair_item<5, ILP, true, false, RP_WIN_WIDE>(A, s, tb, part, bars, phase); break;
                case 6: ok = pair_item<6, ILP, true, false, RP_WIN_WIDE>(A, s, tb, part, bars, phase); break;
                default: ok = pair_item<0, ILP, true, false, RP_WIN_WIDE>(A, s, tb, part, bars, phase); break;
            }
        } else {
            switch (deg) {
                case 3: ok = pair_item<3, ILP, false, false, RP_WIN_WIDE>(A, s, tb, part, bars, phase); break;
                case 4: ok = pair_item<4, ILP, false, false, RP_WIN_WIDE>(A, s, tb, part, bars, phase); break;
                case 5: ok = pair_item<5, ILP, false, false, RP_WIN_WIDE>(A, s, tb, part, bars, phase); break;
                case 6: ok = pair_item<6, ILP, false, false, RP_WIN_WIDE>(A, s, tb, part, bars, phase); break;
                default: ok = pair_item<0, ILP, false, false, RP_WIN_WIDE>(A, s, tb, part, bars, phase); break;
            }
        }
        if (!ok) break;
    }
    RP_PAIR_SMEM_END
}

// Multi-job pair kernel for one (sinc degree, frame kind), with the group's
// jobs in the parameter space: grid row blockIdx.y is job j, so the job
// index is uniform and the scene constants come from the parameter bank.
// One variant per kernel: the 10-way dispatch of k_pairs32m is what makes
// its body spill (~900 bytes a thread; ~50 here).  Every job gets a
// full-width row of blocks; the rows of finished jobs exit at once.
template <int NT, bool ORTHO, int ILP>
__global__ void __launch_bounds__(RP_PAIR_THREADS, 2)
k_pairs32mk(const __grid_constant__ PairJobTable T, unsigned int* work) {
    RP_PAIR_SMEM_DECL
    const int j = blockIdx.y;
    const PairArgs& A = T.job[j].a;
    const unsigned int items = (unsigned)A.nb * A.tblocks * RP_PARTS;
    unsigned int* const wk = work + T.wi[j];
    for (;;) {
        if (tid == 0) s_item = atomicAdd(wk, 1u);
        __syncthreads();
        const unsigned int item = s_item;
        __syncthreads();
        if (item >= items) break;
        const int part = item % RP_PARTS;
        const int tb = (item / RP_PARTS) % A.tblocks;
        const int s = item / (RP_PARTS * A.tblocks);
        if (!pair_item<NT, ILP, ORTHO, false, RP_WIN_WIDE>(A, s, tb, part, bars, phase)) break;
    }
    RP_PAIR_SMEM_END
}

template <int ILP>
void (*pick_mk(int deg, bool ortho))(const PairJobTable, unsigned int*) {
    if (ortho) {
        switch (deg) {
            case 3: return k_pairs32mk<3, true, ILP>;
            case 4: return k_pairs32mk<4, true, ILP>;
            case 5: return k_pairs32mk<5, true, ILP>;
            case 6: return k_pairs32mk<6, true, ILP>;
            default: return k_pairs32mk<0, true, ILP>;
        }
    }
    switch (deg) {
        case 3: return k_pairs32mk<3, false, ILP>;
        case 4: return k_pairs32mk<4, false, ILP>;
        case 5: return k_pairs32mk<5, false, ILP>;
        case 6: return k_pairs32mk<6, false, ILP>;
        default: return k_pairs32mk<0, false, ILP>;
    }
}

int launch_pairs_multik(int cfg, const PairJob* h_jobs, int njobs, unsigned int* work, int sms, cudaStream_t st,
                        const cudaStream_t* aux, int naux) {
    const size_t smem = pair_smem_bytes(RP_WIN_WIDE);
    std::vector<char> done(njobs, 0);
    int nl = 0;     // launches so far (stream round robin)
    for (int a = 0; a < njobs; ++a) {
        if (done[a]) continue;
        const int deg = h_jobs[a].deg;
        const bool ortho = h_jobs[a].ortho != 0;
        auto mk = (cfg & 1) ? pick_mk<4>(deg, ortho) : pick_mk<3>(deg, ortho);
        if (int rc = rp_allow_dyn_smem((const void*)mk, smem)) return rc;
        int occ = 0;
        RP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, mk, RP_PAIR_THREADS, smem));
        // the jobs of this kind, RP_MAXJ per launch
        PairJobTable T;
        int n = 0;
        for (int b = a; b <= njobs; ++b) {
            const bool take = b < njobs && !done[b] && h_jobs[b].deg == deg && (h_jobs[b].ortho != 0) == ortho;
            if (take) {
                T.job[n] = h_jobs[b];
                T.wi[n] = b;
                done[b] = 1;
                ++n;
            }
            if (n > 0 && (n == RP_MAXJ || b == njobs)) {
                T.njobs = n;
                const cudaStream_t ls = naux > 0 ? aux[nl % naux] : st;
                mk<<<dim3((unsigned)(std::max(occ, 1) * sms), (unsigned)n), RP_PAIR_THREADS, smem, ls>>>(T, work);
                RP_CUDA(cudaGetLastError());
                ++nl;
                n = 0;
            }
        }
    }
    return RP_OK;
}

// Configurations (facet pairs per step x resident blocks per SM).  The job's
// scene constants take registers here (the single-batch kernel reads them
// from the parameter bank), so at 2 blocks per SM the body spills ~900
// bytes a thread; at 1 block per SM it fits in 255 registers.
void (*pick_multi(int cfg))(const PairJob*, const unsigned int*, int, unsigned int*) {
    switch (cfg) {
        case 1: return k_pairs32m<3, 1>;
        case 2: return k_pairs32m<3, 2>;
        case 3: return k_pairs32m<4, 2>;
        default: return k_pairs32m<4, 1>;
    }
}

int launch_pairs_multi(int cfg, const PairJob* d_jobs, const unsigned int* d_start, int njobs,
                       unsigned int* d_work, int64_t items, int sms, cudaStream_t st) {
    const size_t smem = pair_smem_bytes(RP_WIN_WIDE);
    auto mk = pick_multi(cfg);
    if (int rc = rp_allow_dyn_smem((const void*)mk, smem)) return rc;
    int occ = 0;
    RP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, mk, RP_PAIR_THREADS, smem));
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)std::max(occ, 1) * sms, items));
    mk<<<grid, RP_PAIR_THREADS, smem, st>>>(d_jobs, d_start, njobs, d_work);
    return RP_OK;
}

}  // namespace rpk
