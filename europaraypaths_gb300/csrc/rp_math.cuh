// rp_math.cuh -- device helpers: reference physics (templated on precision),
// deterministic fixed-point accumulation, and a block-level FFT.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "rp_internal.h"

template <class R> struct Cx { R x, y; };

template <class R> __device__ __forceinline__ Cx<R> cmul(Cx<R> a, Cx<R> b) {
    return Cx<R>{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <class R> __device__ __forceinline__ Cx<R> cadd(Cx<R> a, Cx<R> b) { return Cx<R>{a.x + b.x, a.y + b.y}; }
template <class R> __device__ __forceinline__ Cx<R> csub(Cx<R> a, Cx<R> b) { return Cx<R>{a.x - b.x, a.y - b.y}; }
template <class R> __device__ __forceinline__ Cx<R> cscale(Cx<R> a, R s) { return Cx<R>{a.x * s, a.y * s}; }
template <class R> __device__ __forceinline__ Cx<R> cconj(Cx<R> a) { return Cx<R>{a.x, -a.y}; }

// ---------------------------------------------------------------- physics --
// FP64 restatements used by the plain form and the per-facet precompute.

// elementary_kernels.cu:50-53 -- sinc(x) = sin(pi x)/(pi x), 1 near 0.
__device__ __forceinline__ double d_sinc(double x) {
    if (fabs(x) < 1e-6) return 1.0;
    return sin(RP_PI * x) / (RP_PI * x);
}

// radar_kernels.cu:658-677 -- facet directivity (pi enters the argument twice).
__device__ __forceinline__ double d_facet_G(double th, double ph, double lam, double fs) {
    double piLlam = (RP_PI_F * fs) / lam;
    double st = sin(th);
    double s1 = d_sinc(piLlam * st * cos(ph));
    double s2 = d_sinc(piLlam * st * sin(ph));
    double D = (s1 * s2) * (s1 * s2);
    return D * (4 * RP_PI_F * fs * fs) / (lam * lam);
}

// geometry_kernels.cu:410-412
__device__ __forceinline__ double d_friis(double P, double Gt, double Gr, double lam, double d) {
    return (P * lam * lam * Gt * Gr) / ((4 * RP_PI_FRIIS) * (4 * RP_PI_FRIIS) * d * d);
}

// facetReradiation, geometry_kernels.cu:353-381 (sinc arguments without pi).
__device__ __forceinline__ double d_facet_rerad(double th, double ph, double lam, double fs) {
    double st = sin(th);
    double s1 = d_sinc((fs / lam) * st * cos(ph));
    double s2 = d_sinc((fs / lam) * st * sin(ph));
    double v = (fs * fs / lam) * s1 * s2;
    return v * v;
}

// snellsLaw, geometry_kernels.cu:490-501 (1e4 flags total internal reflection).
__device__ __forceinline__ double d_snells(double th, double e1, double e2) {
    double sR = sqrt(e1 / e2) * sin(th);
    return sR > 1.0 ? 1e4 : asin(sR);
}

// geometry_kernels.cu:384-393
__device__ __forceinline__ double d_radar_eq(double P, double G, double fs, double lam, double d, double nf) {
    double num = P * G * G * fs * fs * fs * fs;
    double den = (4 * RP_PI_FRIIS) * (4 * RP_PI_FRIIS) * d * d * d * d;
    return nf * (num / den);
}

// radar_kernels.cu:167-189
__device__ __forceinline__ double d_rerad(int f, double th1) {
    switch (f) {
        case 0: return 1.0;
        case 1: return th1 * (180 / RP_PI_F) < 1 ? 1.0 : 0.0;
        case 2: return th1 * (180 / RP_PI_F) < 0.5 ? 1.0 : 0.0;
        case 3: return th1 * (RP_PI_F / 180) < 3 ? 1.0 : 0.0;
        case 4: { double s = RP_PI_F / 180; return exp(-0.5 * th1 * th1 / (s * s)); }
        default: return 1.0;
    }
}

__device__ __forceinline__ double clamp1(double x) { return fmax(-1.0, fmin(1.0, x)); }

// prismIntersectionDistance, geometry_kernels.cu:207-269 (FP64).
__device__ inline double d_prism_dist(double ox, double oy, double oz, double dx, double dy,
                                      double dz, const double* box /* xmin,ymin,zmin,xmax,ymax,zmax */,
                                      double t) {
    const double INF = 1e30;
    double o[3] = {ox, oy, oz}, d[3] = {dx, dy, dz};
    double te = -INF, tx = INF;
    for (int a = 0; a < 3; ++a) {
        double mn = box[a], mx = box[a + 3];
        double lo, hi;
        if (fabs(d[a]) < 1e-12) {
            if (o[a] < mn || o[a] > mx) return 0.0;
            lo = -INF; hi = INF;
        } else {
            lo = (mn - o[a]) / d[a];
            hi = (mx - o[a]) / d[a];
            if (lo > hi) { double tmp = lo; lo = hi; hi = tmp; }
        }
        te = fmax(te, lo);
        tx = fmin(tx, hi);
    }
    if (te < 0.0) te = 0.0;
    if (tx > t) tx = t;
    if (te >= tx) return 0.0;
    return tx - te;
}

// ------------------------------------------------- fixed-point accumulation --
// Integer addition is associative, so int64 atomics give a result that does
// not depend on the order in which threads arrive.
__device__ __forceinline__ void fix_add(long long* p, double v, double scale) {
    atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)(long long)llrint(v * scale));
}

// Positive doubles order like their bit patterns: atomicMax on bits.
__device__ __forceinline__ void atomic_max_pos(unsigned long long* p, double v) {
    atomicMax(p, (unsigned long long)__double_as_longlong(v));
}

// ---------------------------------------------------------------- FFT ------
// Block-cooperative radix-2 Stockham FFT on a buffer of n = 2^log2n complex
// values (shared or global memory).  Forward uses e^{-2 pi i k/n}, inverse
// e^{+2 pi i k/n}, unscaled (the cuFFT conventions of the reference).
// tw[k] = e^{-2 pi i k/n} for k < n/2.  The result lands in a or b; the
// returned pointer says which.  Every thread of the block must call it.
template <class R>
__device__ Cx<R>* block_fft(Cx<R>* a, Cx<R>* b, int log2n, int sign, const Cx<R>* tw) {
    const int n = 1 << log2n;
    const int half = n >> 1;
    for (int s = 0; s < log2n; ++s) {
        const int Ns = 1 << s;
        const int step = half >> s;            // n / (2 Ns)
        for (int j = threadIdx.x; j < half; j += blockDim.x) {
            Cx<R> v0 = a[j], v1 = a[j + half];
            int jm = j & (Ns - 1);
            Cx<R> w = tw[jm * step];
            if (sign > 0) w.y = -w.y;
            v1 = cmul(v1, w);
            int o = ((j - jm) << 1) + jm;
            b[o] = cadd(v0, v1);
            b[o + Ns] = csub(v0, v1);
        }
        __syncthreads();
        Cx<R>* t = a; a = b; b = t;
    }
    return a;
}

// Bluestein DFT of length N (not a power of two) via power-of-two length M.
//   x:   input/output, N values (overwritten with the transform)
//   wa, wb: work buffers of M values each
//   bw:  w_k = e^{-i pi k^2 / N} (N values); bW: FFT_M of the conj chirp
//   sign: -1 forward, +1 inverse (unscaled)
template <class R>
__device__ void block_bluestein(Cx<R>* x, Cx<R>* wa, Cx<R>* wb, int N, int log2M, int sign,
                                const Cx<R>* bw, const Cx<R>* bW, const Cx<R>* twM) {
    const int M = 1 << log2M;
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        Cx<R> v{R(0), R(0)};
        if (k < N) {
            Cx<R> w = bw[k];
            if (sign > 0) w.y = -w.y;
            v = cmul(x[k], w);
        }
        wa[k] = v;
    }
    __syncthreads();
    Cx<R>* y = block_fft<R>(wa, wb, log2M, -1, twM);
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        Cx<R> W = (sign < 0) ? bW[k] : cconj(bW[(M - k) & (M - 1)]);
        y[k] = cmul(y[k], W);
    }
    __syncthreads();
    Cx<R>* other = (y == wa) ? wb : wa;
    Cx<R>* z = block_fft<R>(y, other, log2M, +1, twM);
    const R inv = R(1) / R(M);
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        Cx<R> w = bw[k];
        if (sign > 0) w.y = -w.y;
        x[k] = cscale(cmul(z[k], w), inv);
    }
    __syncthreads();
}

// Device view of a DftPlan in precision R.
template <class R> struct PlanV {
    int n, pow2, log2M;
    const Cx<R>* tw;
    const Cx<R>* bw;
    const Cx<R>* bW;
};

inline PlanV<double> plan_view64(const DftPlan& p) {
    return PlanV<double>{p.n, p.pow2, p.log2M, (const Cx<double>*)p.tw64,
                         (const Cx<double>*)p.bw64, (const Cx<double>*)p.bW64};
}
inline PlanV<float> plan_view32(const DftPlan& p) {
    return PlanV<float>{p.n, p.pow2, p.log2M, (const Cx<float>*)p.tw32,
                        (const Cx<float>*)p.bw32, (const Cx<float>*)p.bW32};
}

// DFT of length pl.n of the values in x (x, wa, wb each hold M values).
// Returns the buffer holding the n results (x or wa for a power of two,
// x for Bluestein).  sign -1 forward, +1 inverse (unscaled).
template <class R>
__device__ Cx<R>* block_dft(Cx<R>* x, Cx<R>* wa, Cx<R>* wb, const PlanV<R>& pl, int sign) {
    if (pl.pow2) return block_fft<R>(x, wa, pl.log2M, sign, pl.tw);
    block_bluestein<R>(x, wa, wb, pl.n, pl.log2M, sign, pl.bw, pl.bW, pl.tw);
    return x;
}

// Incoherent mode's surface phase, in turns: a counter-based hash of (seed,
// the source position's bits, the facet's index in the scene's input order)
// made of the SplitMix64 mixing function (Steele, Lea, Flood 2014), its top
// 24 bits as k / 2^24.  The reference draws the phase from clock64()
// (randomPhasor, radar_kernels.cu:689-711), which no run reproduces.
__host__ __device__ __forceinline__ uint64_t rp_mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t rp_dbits(double v) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(v);
#else
    uint64_t u;
    memcpy(&u, &v, sizeof(u));
    return u;
#endif
}
__host__ __device__ __forceinline__ double rp_incoherent_turns(uint64_t seed, double sx, double sy, double sz,
                                                               int64_t facet) {
    const uint64_t key = rp_mix64(rp_mix64(rp_mix64(rp_mix64(seed) ^ rp_dbits(sx)) ^ rp_dbits(sy)) ^ rp_dbits(sz));
    return (double)(rp_mix64(key ^ (uint64_t)facet) >> 40) * (1.0 / 16777216.0);
}

