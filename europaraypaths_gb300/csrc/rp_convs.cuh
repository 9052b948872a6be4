// rp_convs.cuh -- the shared-memory range compression (k_conv32s, rp_convs.cu):
// its job arguments and launch entry point.
#pragma once

#include "rp_fft.cuh"
#include "rp_internal.h"
#include "rp_pair.cuh"

#define RP_CONV_SPLIT 64       // targets per range-compression work item (fixed:
                               // a trace's sum order never depends on the batch)
#define RP_CONV_THREADS 512

namespace rpk {

// Arguments of one segment's range compression (a job of k_conv32s): the
// targets' rows T (and T2), their windows, the target chirp's spectrum C2s
// and the crop kernel's Hs (both in the in-place transforms' digit-reversed
// order), and the per-split sums of u it writes (radar_kernels.cu:554-649,
// elementary_kernels.cu:258-353).
struct ConvArgs {
    const int* ntl;
    int64_t tstride;
    int nb;
    const int* bt0;
    const C32* T;           // rows [RP_PARTS][nb][tstride][Wt], each element {high, low}
    const C32* T2;          // specular mode: the outbound leg's parts (Psour), else null
    int Wt;
    const Cplx<float>* C2s;
    const Cplx<float>* Hs;  // DIF_M(crop kernel) / M
    int nr, n2, N, M, crop_K, crop_all;
    float sig_scale;
    C32* part;          // [nb][nsplit][n2]: per split, the targets' sum of u
    int nsplit;
    unsigned int* work;
};

// The length class of a job of storage mode `mode` with transform length n2
// = 2nr: n2 itself for the lengths that have a kernel of their own, else 0
// (the kernel that reads the length at run time).
int conv_length_class(int mode, int n2);

// One compression launch over a job table of one storage mode and length
// class nc (0: several lengths) (mode 0: X, W and U in shared memory; 1: X
// parked in global scratch; 2: sub-blocks of the transforms in shared
// memory, the rest in global scratch); modes 1 and 2 take at most `slots`
// blocks, one per slot of the global scratch.  spec: the table's segments
// are specular.
int launch_conv32s(const ConvArgs* d_jobs, const unsigned int* d_start, int njobs, int mode, int nc,
                   size_t csm, int sms, int slots, unsigned int items, unsigned int* work, C32* gscr,
                   size_t gslot, bool spec, cudaStream_t st);

}  // namespace rpk
