// rp_conv.cuh -- block-level range compression: the linear chirp convolution
// of convolvePhasorChirpLinear (radar_kernels.cu:554-649) and the cropped,
// decimated complex convolution of convolveComplex (elementary_kernels.cu:
// 258-353), for one trace per thread block, in precision R.
#pragma once

#include "rp_math.cuh"

// out[i] = (1/2nr) * IDFT_2nr( DFT_2nr(pad(in)) * C )[nr/2 + i],  i < nr.
// x, wa, wb: scratch of pl.M() values each.  `in` may alias `out`.
template <class R>
__device__ void conv_linear_block(const Cx<R>* in, const Cx<R>* C, const PlanV<R>& pl, int nr,
                                  Cx<R>* x, Cx<R>* wa, Cx<R>* wb, Cx<R>* out, R extra_scale) {
    const int L = pl.n;                 // 2 nr
    const int M = 1 << pl.log2M;
    for (int k = threadIdx.x; k < M; k += blockDim.x)
        x[k] = (k < nr) ? in[k] : Cx<R>{R(0), R(0)};
    __syncthreads();
    Cx<R>* r = block_dft<R>(x, wa, wb, pl, -1);
    for (int k = threadIdx.x; k < L; k += blockDim.x) r[k] = cmul(r[k], C[k]);
    __syncthreads();
    Cx<R>* a2 = (r == x) ? wa : x;
    Cx<R>* r2 = block_dft<R>(r, a2, wb, pl, +1);
    const R sc = extra_scale / R(L);
    const int h = nr / 2;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) out[i] = cscale(r2[h + i], sc);
    __syncthreads();
}

// out[k] = (1/N) IDFT_N( DFT_N(pad sig) * crop(DFT_N(pad ker)) )[2k], k < nr,
// N = 2 nr - 1; crop zeroes bins with min(k, N-k) > K (|freq| > B).
// A, B, wa, wb: scratch of pl.M() values each.  N is odd, so pl is Bluestein.
template <class R>
__device__ void conv_complex_block(const Cx<R>* sig, const Cx<R>* ker, const PlanV<R>& pl, int nr,
                                   int crop_K, int crop_all, Cx<R>* A, Cx<R>* B, Cx<R>* wa,
                                   Cx<R>* wb, Cx<R>* out, R extra_scale) {
    const int N = pl.n;
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        A[k] = (k < nr) ? sig[k] : Cx<R>{R(0), R(0)};
        B[k] = (k < nr) ? ker[k] : Cx<R>{R(0), R(0)};
    }
    __syncthreads();
    block_dft<R>(A, wa, wb, pl, -1);
    block_dft<R>(B, wa, wb, pl, -1);
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        int m = k < N - k ? k : N - k;
        bool keep = crop_all || m <= crop_K;
        A[k] = keep ? cmul(A[k], B[k]) : Cx<R>{R(0), R(0)};
    }
    __syncthreads();
    block_dft<R>(A, wa, wb, pl, +1);
    const R sc = extra_scale / R(N);
    for (int k = threadIdx.x; k < nr; k += blockDim.x) out[k] = cscale(A[2 * k], sc);
    __syncthreads();
}

// out[i] = (1/nr) IDFT_nr( DFT_nr(in) * C )[i]: the circular convolution of
// convolvePhasorChirp (radar_kernels.cu:516-552).  x, wa, wb: scratch of
// pl.M() values each.  `in` may alias `out`.
template <class R>
__device__ void conv_circular_block(const Cx<R>* in, const Cx<R>* C, const PlanV<R>& pl, int nr,
                                    Cx<R>* x, Cx<R>* wa, Cx<R>* wb, Cx<R>* out) {
    const int M = 1 << pl.log2M;
    for (int k = threadIdx.x; k < M; k += blockDim.x)
        x[k] = (k < nr) ? in[k] : Cx<R>{R(0), R(0)};
    __syncthreads();
    Cx<R>* r = block_dft<R>(x, wa, wb, pl, -1);
    for (int k = threadIdx.x; k < nr; k += blockDim.x) r[k] = cmul(r[k], C[k]);
    __syncthreads();
    Cx<R>* a2 = (r == x) ? wa : x;
    Cx<R>* r2 = block_dft<R>(r, a2, wb, pl, +1);
    const R sc = R(1) / R(nr);
    for (int i = threadIdx.x; i < nr; i += blockDim.x) out[i] = cscale(r2[i], sc);
    __syncthreads();
}
