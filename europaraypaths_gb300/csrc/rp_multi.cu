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

// Estimated duration of one work item of a job: its facet-part capacity
// times the targets of a full target block (host bounds of the wave).
static double item_cost(const PairJob& j) {
    const double tpb = (double)std::min<int64_t>(j.a.tstride, RP_PAIR_THREADS);
    return (double)j.a.rstride / RP_PARTS * tpb;
}

int launch_pairs_multik(int cfg, const PairJob* h_jobs, int njobs, unsigned int* work, int sms, cudaStream_t st,
                        const cudaStream_t* aux, int naux) {
    const size_t smem = pair_smem_bytes(RP_WIN_WIDE);
    // the (sinc degree, frame kind) groups, each's jobs by decreasing item
    // cost: a launch's blocks take its jobs in order, so the launch ends on
    // the jobs with the shortest items, not on a large scene's last items;
    // the groups with the most work are launched first
    struct Kind { int deg; bool ortho; double work; std::vector<int> jobs; };
    std::vector<Kind> kinds;
    for (int b = 0; b < njobs; ++b) {
        const int deg = h_jobs[b].deg;
        const bool ortho = h_jobs[b].ortho != 0;
        size_t k = 0;
        while (k < kinds.size() && !(kinds[k].deg == deg && kinds[k].ortho == ortho)) ++k;
        if (k == kinds.size()) kinds.push_back(Kind{deg, ortho, 0.0, {}});
        kinds[k].jobs.push_back(b);
        kinds[k].work += item_cost(h_jobs[b]) * (double)h_jobs[b].a.nb * h_jobs[b].a.tblocks;
    }
    std::stable_sort(kinds.begin(), kinds.end(), [](const Kind& x, const Kind& y) { return x.work > y.work; });
    int nl = 0;     // launches so far (stream round robin)
    for (Kind& K : kinds) {
        std::stable_sort(K.jobs.begin(), K.jobs.end(),
                         [&](int x, int y) { return item_cost(h_jobs[x]) > item_cost(h_jobs[y]); });
        auto mk = (cfg & 1) ? pick_mk<4>(K.deg, K.ortho) : pick_mk<3>(K.deg, K.ortho);
        if (int rc = rp_allow_dyn_smem((const void*)mk, smem)) return rc;
        int occ = 0;
        RP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, mk, RP_PAIR_THREADS, smem));
        // the kind's jobs, RP_MAXJ per launch
        for (size_t j0 = 0; j0 < K.jobs.size(); j0 += RP_MAXJ) {
            PairJobTable T;
            const int n = (int)std::min<size_t>(RP_MAXJ, K.jobs.size() - j0);
            for (int i = 0; i < n; ++i) {
                T.job[i] = h_jobs[K.jobs[j0 + i]];
                T.wi[i] = K.jobs[j0 + i];
            }
            T.njobs = n;
            const cudaStream_t ls = naux > 0 ? aux[nl % naux] : st;
            mk<<<dim3((unsigned)(std::max(occ, 1) * sms), (unsigned)n), RP_PAIR_THREADS, smem, ls>>>(T, work);
            RP_CUDA(cudaGetLastError());
            ++nl;
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
