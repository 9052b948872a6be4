// rp_fft.cuh -- in-place power-of-two FFT stages shared by the host (table
// preparation) and the device (block-level transforms in shared memory).
//
// Forward transforms are decimation-in-frequency: natural order in,
// digit-reversed order out.  Inverse transforms are the mirrored
// decimation-in-time stages: digit-reversed in, natural out, unscaled
// (DIT(DIF(x)) = n x, the cuFFT convention of the reference).  Pointwise
// products between two DIF outputs of the same length are therefore valid in
// the scrambled order, and no permutation pass is ever needed.  Spectral
// tables (chirp and Bluestein kernels) are prepared on the host with these
// same stage functions, so they come out in the device's order.
//
// Stage schedule for n = 2^m: DIF runs radix-4 stages of span L = n, n/4,
// ... while L >= 4, then one radix-2 stage (L = 2) if m is odd; DIT runs the
// same stages in reverse.  Twiddles come from a table tw[k] = e^{-2 pi i k/M}
// of a power of two M >= n (k < M): e^{-2 pi i j/L} = tw[j * (M / L)].
#pragma once

#include <cuda_runtime.h>

template <class T> struct Cplx { T x, y; };

template <class T> __host__ __device__ __forceinline__ Cplx<T> c_mul(Cplx<T> a, Cplx<T> b) {
    return Cplx<T>{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <class T> __host__ __device__ __forceinline__ Cplx<T> c_mulc(Cplx<T> a, Cplx<T> b) {
    // a * conj(b)
    return Cplx<T>{a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}
template <class T> __host__ __device__ __forceinline__ Cplx<T> c_add(Cplx<T> a, Cplx<T> b) { return Cplx<T>{a.x + b.x, a.y + b.y}; }
template <class T> __host__ __device__ __forceinline__ Cplx<T> c_sub(Cplx<T> a, Cplx<T> b) { return Cplx<T>{a.x - b.x, a.y - b.y}; }

__host__ __device__ __forceinline__ int fft_log2(int n) {
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}

// One radix-4 DIF butterfly, t in [0, n/4), stage span L (L >= 4).
template <class T, class TW>
__host__ __device__ __forceinline__ void dif4(Cplx<T>* a, int L, int lq, int t, const TW& tw, int mshift) {
    const int q4 = L >> 2;
    const int j = t & (q4 - 1);
    const int b = (t >> lq) * L + j;       // lq = log2(q4)
    Cplx<T> x0 = a[b], x1 = a[b + q4], x2 = a[b + 2 * q4], x3 = a[b + 3 * q4];
    Cplx<T> t0 = c_add(x0, x2), t1 = c_sub(x0, x2), t2 = c_add(x1, x3), t3 = c_sub(x1, x3);
    Cplx<T> y0 = c_add(t0, t2), y2 = c_sub(t0, t2);
    Cplx<T> y1 = Cplx<T>{t1.x + t3.y, t1.y - t3.x};   // t1 - i t3
    Cplx<T> y3 = Cplx<T>{t1.x - t3.y, t1.y + t3.x};   // t1 + i t3
    a[b] = y0;
    if (j == 0) {
        a[b + q4] = y1; a[b + 2 * q4] = y2; a[b + 3 * q4] = y3;
    } else {
        Cplx<T> w1 = tw(j << mshift);              // e^{-2 pi i j / L}
        Cplx<T> w2 = c_mul(w1, w1);
        Cplx<T> w3 = c_mul(w1, w2);
        a[b + q4] = c_mul(y1, w1);
        a[b + 2 * q4] = c_mul(y2, w2);
        a[b + 3 * q4] = c_mul(y3, w3);
    }
}

// One radix-4 DIT butterfly (inverse direction), mirror of dif4.
template <class T, class TW>
__host__ __device__ __forceinline__ void dit4(Cplx<T>* a, int L, int lq, int t, const TW& tw, int mshift) {
    const int q4 = L >> 2;
    const int j = t & (q4 - 1);
    const int b = (t >> lq) * L + j;
    Cplx<T> x0 = a[b], x1 = a[b + q4], x2 = a[b + 2 * q4], x3 = a[b + 3 * q4];
    if (j != 0) {
        Cplx<T> w1 = tw(j << mshift);
        Cplx<T> w2 = c_mul(w1, w1);
        Cplx<T> w3 = c_mul(w1, w2);
        x1 = c_mulc(x1, w1);
        x2 = c_mulc(x2, w2);
        x3 = c_mulc(x3, w3);
    }
    Cplx<T> t0 = c_add(x0, x2), t1 = c_sub(x0, x2), t2 = c_add(x1, x3), t3 = c_sub(x1, x3);
    a[b] = c_add(t0, t2);
    a[b + 2 * q4] = c_sub(t0, t2);
    a[b + q4] = Cplx<T>{t1.x - t3.y, t1.y + t3.x};       // t1 + i t3
    a[b + 3 * q4] = Cplx<T>{t1.x + t3.y, t1.y - t3.x};   // t1 - i t3
}

// Radix-2 stages of span L (t in [0, n/2)).
template <class T, class TW>
__host__ __device__ __forceinline__ void dif2(Cplx<T>* a, int L, int lh, int t, const TW& tw, int mshift) {
    const int h = L >> 1;
    const int j = t & (h - 1);
    const int b = (t >> lh) * L + j;
    Cplx<T> x0 = a[b], x1 = a[b + h];
    a[b] = c_add(x0, x1);
    Cplx<T> d = c_sub(x0, x1);
    a[b + h] = (j == 0) ? d : c_mul(d, tw(j << mshift));
}

template <class T, class TW>
__host__ __device__ __forceinline__ void dit2(Cplx<T>* a, int L, int lh, int t, const TW& tw, int mshift) {
    const int h = L >> 1;
    const int j = t & (h - 1);
    const int b = (t >> lh) * L + j;
    Cplx<T> x0 = a[b], x1 = a[b + h];
    if (j != 0) x1 = c_mulc(x1, tw(j << mshift));
    a[b] = c_add(x0, x1);
    a[b + h] = c_sub(x0, x1);
}

// Host: full transforms (serial), used to prepare device-order tables.
template <class T, class TW>
void host_dif(Cplx<T>* a, int n, const TW& tw, int log2M) {
    const int m = fft_log2(n);
    int L = n, lL = m;
    for (; L >= 4; L >>= 2, lL -= 2)
        for (int t = 0; t < n / 4; ++t) dif4(a, L, lL - 2, t, tw, log2M - lL);
    if (L == 2)
        for (int t = 0; t < n / 2; ++t) dif2(a, 2, 0, t, tw, log2M - 1);
}

template <class T, class TW>
void host_dit(Cplx<T>* a, int n, const TW& tw, int log2M) {
    const int m = fft_log2(n);
    int L, lL;
    if (m & 1) {
        for (int t = 0; t < n / 2; ++t) dit2(a, 2, 0, t, tw, log2M - 1);
        L = 8; lL = 3;
    } else {
        L = 4; lL = 2;
    }
    for (; L <= n; L <<= 2, lL += 2)
        for (int t = 0; t < n / 4; ++t) dit4(a, L, lL - 2, t, tw, log2M - lL);
}

#ifdef __CUDACC__
// Device: block-cooperative transforms on shared memory; every thread of the
// block must call them.  tw reads the global twiddle table of length M.
template <class T, class TW>
__device__ void block_dif(Cplx<T>* a, int n, const TW& tw, int log2M) {
    const int m = fft_log2(n);
    int L = n, lL = m;
    for (; L >= 4; L >>= 2, lL -= 2) {
        for (int t = threadIdx.x; t < n / 4; t += blockDim.x) dif4(a, L, lL - 2, t, tw, log2M - lL);
        __syncthreads();
    }
    if (L == 2) {
        for (int t = threadIdx.x; t < n / 2; t += blockDim.x) dif2(a, 2, 0, t, tw, log2M - 1);
        __syncthreads();
    }
}

template <class T, class TW>
__device__ void block_dit(Cplx<T>* a, int n, const TW& tw, int log2M) {
    const int m = fft_log2(n);
    int L, lL;
    if (m & 1) {
        for (int t = threadIdx.x; t < n / 2; t += blockDim.x) dit2(a, 2, 0, t, tw, log2M - 1);
        __syncthreads();
        L = 8; lL = 3;
    } else {
        L = 4; lL = 2;
    }
    for (; L <= n; L <<= 2, lL += 2) {
        for (int t = threadIdx.x; t < n / 4; t += blockDim.x) dit4(a, L, lL - 2, t, tw, log2M - lL);
        __syncthreads();
    }
}

// Fused radix-4 stage pairs ("radix 16", used by block_dif_s / block_dit_s
// below): the 16 elements a[base + i*S], i < 16, are closed under two
// consecutive radix-4 stages (DIF spans L, L/4 with S = L/16; DIT spans L,
// 4L with S = L/4), so one thread keeps them in registers across both and a
// transform makes about half the passes over shared memory (and half the
// barriers).  The stage schedule is the one of block_dif / block_dit above,
// so outputs keep the same digit-reversed order.  Twiddles are applied
// unconditionally (tw(0) = 1 exactly).
template <class T>
__device__ __forceinline__ void r4_dif_reg(Cplx<T>& x0, Cplx<T>& x1, Cplx<T>& x2, Cplx<T>& x3, Cplx<T> w1) {
    const Cplx<T> t0 = c_add(x0, x2), t1 = c_sub(x0, x2), t2 = c_add(x1, x3), t3 = c_sub(x1, x3);
    const Cplx<T> y1 = Cplx<T>{t1.x + t3.y, t1.y - t3.x};
    const Cplx<T> y3 = Cplx<T>{t1.x - t3.y, t1.y + t3.x};
    const Cplx<T> w2 = c_mul(w1, w1), w3 = c_mul(w1, w2);
    x0 = c_add(t0, t2);
    x1 = c_mul(y1, w1);
    x2 = c_mul(c_sub(t0, t2), w2);
    x3 = c_mul(y3, w3);
}

template <class T>
__device__ __forceinline__ void r4_dit_reg(Cplx<T>& x0, Cplx<T>& x1, Cplx<T>& x2, Cplx<T>& x3, Cplx<T> w1) {
    const Cplx<T> w2 = c_mul(w1, w1), w3 = c_mul(w1, w2);
    const Cplx<T> v1 = c_mulc(x1, w1), v2 = c_mulc(x2, w2), v3 = c_mulc(x3, w3);
    const Cplx<T> t0 = c_add(x0, v2), t1 = c_sub(x0, v2), t2 = c_add(v1, v3), t3 = c_sub(v1, v3);
    x0 = c_add(t0, t2);
    x2 = c_sub(t0, t2);
    x1 = Cplx<T>{t1.x - t3.y, t1.y + t3.x};
    x3 = Cplx<T>{t1.x + t3.y, t1.y - t3.x};
}

#endif

#ifdef __CUDACC__
// Swizzled variants for the compression kernel.  Element e of a shared
// array lives at swz(e) = e ^ (2 ((e >> 5) & 15)): a permutation inside each
// row of 32 complex values that XORs the column with twice the row index.
// The fused passes whose groups stride 2 or 4 elements (lanes in 8 or 4
// consecutive rows) then reach 16 distinct bank pairs per half-warp, and
// the permutation keeps each even-odd pair of elements adjacent (the XOR
// value is even), so a pair moves as one 16-byte access (ld_pair /
// st_pair).  Twiddles e^{-2 pi i j / L} come from the special-function unit
// (__sincosf, |angle| <= pi / 2, absolute error below 1e-6) instead of a
// table.
__device__ __forceinline__ int swz(int e) { return e ^ ((e >> 4) & 30); }

// Elements e and e + 1 (e even) of a swizzled array, 16-byte aligned when a is.
template <class T>
__device__ __forceinline__ void ld_pair(const Cplx<T>* a, int e, Cplx<T>& x0, Cplx<T>& x1) {
    const float4 v = *reinterpret_cast<const float4*>(a + swz(e));
    x0 = Cplx<T>{v.x, v.y};
    x1 = Cplx<T>{v.z, v.w};
}
template <class T>
__device__ __forceinline__ void st_pair(Cplx<T>* a, int e, Cplx<T> x0, Cplx<T> x1) {
    *reinterpret_cast<float4*>(a + swz(e)) = make_float4(x0.x, x0.y, x1.x, x1.y);
}

// The B elements k0 .. k0 + B - 1 (a block of B, k0 = blk B) as B / 2 pair
// accesses.  For B = 4 the lanes whose block index has bit 2 set take their
// second pair first: a quarter-warp's eight 16-byte accesses then cover all
// eight bank groups (in order, blocks 2 chunks apart would meet pairwise).
template <int B, class T>
__device__ __forceinline__ void ld_pairs(const Cplx<T>* a, int k0, Cplx<T> (&x)[B]) {
    if constexpr (B == 4) {
        const bool r = (k0 >> 4) & 1;
        Cplx<T> p0, p1, q0, q1;
        ld_pair(a, k0 + (r ? 2 : 0), p0, p1);
        ld_pair(a, k0 + (r ? 0 : 2), q0, q1);
        x[0] = r ? q0 : p0; x[1] = r ? q1 : p1;
        x[2] = r ? p0 : q0; x[3] = r ? p1 : q1;
    } else {
#pragma unroll
        for (int i = 0; i < B; i += 2) ld_pair(a, k0 + i, x[i], x[i + 1]);
    }
}
template <int B, class T>
__device__ __forceinline__ void st_pairs(Cplx<T>* a, int k0, const Cplx<T> (&x)[B]) {
    if constexpr (B == 4) {
        const bool r = (k0 >> 4) & 1;
        st_pair(a, k0 + (r ? 2 : 0), r ? x[2] : x[0], r ? x[3] : x[1]);
        st_pair(a, k0 + (r ? 0 : 2), r ? x[0] : x[2], r ? x[1] : x[3]);
    } else {
#pragma unroll
        for (int i = 0; i < B; i += 2) st_pair(a, k0 + i, x[i], x[i + 1]);
    }
}

template <class T>
__device__ __forceinline__ Cplx<T> tw_sfu(int j, float step) {   // e^{-i j step}
    float sn, cs;
    __sincosf((float)j * step, &sn, &cs);
    return Cplx<T>{(T)cs, (T)-sn};
}

// The two radix-4 DIF stages of spans L and L/4 on one group's 16 elements
// in registers: x[i] = a[base + i S], S = L / 16, b = base mod S.
template <class T>
__device__ __forceinline__ void dif16_regs(Cplx<T> (&x)[16], int b, int L) {
    const int S = L >> 4;
    const float st1 = 6.28318530717958647f / (float)L, st2 = 4.f * st1;
#pragma unroll
    for (int i = 0; i < 4; ++i) r4_dif_reg(x[i], x[i + 4], x[i + 8], x[i + 12], tw_sfu<T>(b + i * S, st1));
    const Cplx<T> w = tw_sfu<T>(b, st2);
#pragma unroll
    for (int c = 0; c < 4; ++c) r4_dif_reg(x[4 * c], x[4 * c + 1], x[4 * c + 2], x[4 * c + 3], w);
}

// The two radix-4 DIT stages of spans L and 4L on one group's 16 elements in
// registers: x[i] = a[base + i S], S = L / 4, b = base mod S.
template <class T>
__device__ __forceinline__ void dit16_regs(Cplx<T> (&x)[16], int b, int L) {
    const int S = L >> 2;
    const float st1 = 6.28318530717958647f / (float)L, st2 = 0.25f * st1;
    const Cplx<T> w = tw_sfu<T>(b, st1);
#pragma unroll
    for (int c = 0; c < 4; ++c) r4_dit_reg(x[4 * c], x[4 * c + 1], x[4 * c + 2], x[4 * c + 3], w);
#pragma unroll
    for (int k = 0; k < 4; ++k) r4_dit_reg(x[k], x[k + 4], x[k + 8], x[k + 12], tw_sfu<T>(b + k * S, st2));
}

// DIF stages from span L0 down (L0 = n: the whole transform; L0 = n / 16:
// all but the first fused pass, which a caller ran on its own registers).
// Ends with a barrier.
template <class T>
__device__ __forceinline__ void block_dif_s_from(Cplx<T>* a, int n, int L0) {
    int L = L0, lL = fft_log2(L0);
#pragma unroll
    for (; L >= 16; L >>= 4, lL -= 4) {
        const int lS = lL - 4, S = 1 << lS;
        for (int g = threadIdx.x; g < (n >> 4); g += blockDim.x) {
            const int b = g & (S - 1);
            const int base = (g >> lS) * L + b;
            Cplx<T> x[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) x[i] = a[swz(base + i * S)];
            dif16_regs(x, b, L);
#pragma unroll
            for (int i = 0; i < 16; ++i) a[swz(base + i * S)] = x[i];
        }
        __syncthreads();
    }
    if (L >= 4) {   // one remaining radix-4 stage (L = 4 or 8)
        const int q4 = L >> 2, lq = lL - 2;
        const float st = 6.28318530717958647f / (float)L;
        for (int t = threadIdx.x; t < n / 4; t += blockDim.x) {
            const int j = t & (q4 - 1);
            const int b = (t >> lq) * L + j;
            Cplx<T> x0 = a[swz(b)], x1 = a[swz(b + q4)], x2 = a[swz(b + 2 * q4)], x3 = a[swz(b + 3 * q4)];
            r4_dif_reg(x0, x1, x2, x3, tw_sfu<T>(j, st));
            a[swz(b)] = x0; a[swz(b + q4)] = x1; a[swz(b + 2 * q4)] = x2; a[swz(b + 3 * q4)] = x3;
        }
        __syncthreads();
        L >>= 2;
    }
    if (L == 2) {
        for (int t = threadIdx.x; t < n / 2; t += blockDim.x) {
            const Cplx<T> x0 = a[swz(2 * t)], x1 = a[swz(2 * t + 1)];
            a[swz(2 * t)] = c_add(x0, x1);
            a[swz(2 * t + 1)] = c_sub(x0, x1);
        }
        __syncthreads();
    }
}

template <class T>
__device__ __forceinline__ void block_dif_s(Cplx<T>* a, int n) { block_dif_s_from(a, n, n); }

// DIT stages up to the fused passes of span <= Lmax (Lmax = n / 4: the whole
// transform; Lmax = n / 16: all but the last fused pass, spans n / 4 and n,
// which a caller runs on its own registers).  Ends with a barrier when it
// ran any stage.
template <class T>
__device__ __forceinline__ void block_dit_s_upto(Cplx<T>* a, int n, int Lmax) {
    const int m = fft_log2(n);
    int L, lL;
    if (m & 1) {
        for (int t = threadIdx.x; t < n / 2; t += blockDim.x) {
            const Cplx<T> x0 = a[swz(2 * t)], x1 = a[swz(2 * t + 1)];
            a[swz(2 * t)] = c_add(x0, x1);
            a[swz(2 * t + 1)] = c_sub(x0, x1);
        }
        __syncthreads();
        L = 8; lL = 3;
    } else {
        L = 4; lL = 2;
    }
    if ((m >> 1) & 1) {   // an odd number of radix-4 stages: the smallest runs alone
        const int q4 = L >> 2, lq = lL - 2;
        const float st = 6.28318530717958647f / (float)L;
        for (int t = threadIdx.x; t < n / 4; t += blockDim.x) {
            const int j = t & (q4 - 1);
            const int b = (t >> lq) * L + j;
            Cplx<T> x0 = a[swz(b)], x1 = a[swz(b + q4)], x2 = a[swz(b + 2 * q4)], x3 = a[swz(b + 3 * q4)];
            r4_dit_reg(x0, x1, x2, x3, tw_sfu<T>(j, st));
            a[swz(b)] = x0; a[swz(b + q4)] = x1; a[swz(b + 2 * q4)] = x2; a[swz(b + 3 * q4)] = x3;
        }
        __syncthreads();
        L <<= 2;
        lL += 2;
    }
#pragma unroll
    for (; L <= Lmax; L <<= 4, lL += 4) {
        const int lS = lL - 2, S = 1 << lS;
        for (int g = threadIdx.x; g < (n >> 4); g += blockDim.x) {
            const int b = g & (S - 1);
            const int base = (g >> lS) * (4 * L) + b;
            Cplx<T> x[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) x[i] = a[swz(base + i * S)];
            dit16_regs(x, b, L);
#pragma unroll
            for (int i = 0; i < 16; ++i) a[swz(base + i * S)] = x[i];
        }
        __syncthreads();
    }
}

template <class T>
__device__ __forceinline__ void block_dit_s(Cplx<T>* a, int n) { block_dit_s_upto(a, n, n / 4); }

// ---- the edge block: the last DIF stages and the first DIT stages of a
// length-n transform both act within contiguous blocks of B elements, B =
// 16, 2, 4, 8 for log2 n = 0, 1, 2, 3 mod 4 (the last fused DIF pass at span
// 16 and the first fused DIT pass at span 4; the radix-2 stage; the lone
// radix-4 stage at span 4; the radix-4 stage at span 8 with the radix-2
// stage).  So a pointwise product between a forward and an inverse
// transform can sit between them in registers: one pass over the data
// instead of three.  The stage arithmetic is the same as block_dif_s /
// block_dit_s.
__host__ __device__ __forceinline__ int edge_block(int n) {
    const int r = fft_log2(n) & 3;
    return r == 0 ? 16 : (r == 1 ? 2 : (r == 2 ? 4 : 8));
}

template <class T, int B>
__device__ __forceinline__ void dif_edge(Cplx<T> (&x)[B]) {
    if constexpr (B == 16) {
        dif16_regs(x, 0, 16);
    } else if constexpr (B == 8) {
        const float st = 6.28318530717958647f / 8.f;
#pragma unroll
        for (int j = 0; j < 2; ++j) r4_dif_reg(x[j], x[j + 2], x[j + 4], x[j + 6], tw_sfu<T>(j, st));
#pragma unroll
        for (int p = 0; p < 8; p += 2) {
            const Cplx<T> a = x[p], b = x[p + 1];
            x[p] = c_add(a, b);
            x[p + 1] = c_sub(a, b);
        }
    } else if constexpr (B == 4) {
        r4_dif_reg(x[0], x[1], x[2], x[3], tw_sfu<T>(0, 6.28318530717958647f / 4.f));
    } else {
        const Cplx<T> a = x[0], b = x[1];
        x[0] = c_add(a, b);
        x[1] = c_sub(a, b);
    }
}

template <class T, int B>
__device__ __forceinline__ void dit_edge(Cplx<T> (&x)[B]) {
    if constexpr (B == 16) {
        dit16_regs(x, 0, 4);
    } else if constexpr (B == 8) {
#pragma unroll
        for (int p = 0; p < 8; p += 2) {
            const Cplx<T> a = x[p], b = x[p + 1];
            x[p] = c_add(a, b);
            x[p + 1] = c_sub(a, b);
        }
        const float st = 6.28318530717958647f / 8.f;
#pragma unroll
        for (int j = 0; j < 2; ++j) r4_dit_reg(x[j], x[j + 2], x[j + 4], x[j + 6], tw_sfu<T>(j, st));
    } else if constexpr (B == 4) {
        r4_dit_reg(x[0], x[1], x[2], x[3], tw_sfu<T>(0, 6.28318530717958647f / 4.f));
    } else {
        const Cplx<T> a = x[0], b = x[1];
        x[0] = c_add(a, b);
        x[1] = c_sub(a, b);
    }
}

// DIF fused passes of spans L0, L0 / 16, ... > 16: the passes between a
// transform's first pass (span n, run by the caller) and its edge block.
// Ends with a barrier when it ran a pass.
template <class T>
__device__ __forceinline__ void block_dif_s_mid(Cplx<T>* a, int n, int L0) {
#pragma unroll
    for (int L = L0, lL = fft_log2(L0); L > 16; L >>= 4, lL -= 4) {
        const int lS = lL - 4, S = 1 << lS;
        for (int g = threadIdx.x; g < (n >> 4); g += blockDim.x) {
            const int b = g & (S - 1);
            const int base = (g >> lS) * L + b;
            Cplx<T> x[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) x[i] = a[swz(base + i * S)];
            dif16_regs(x, b, L);
#pragma unroll
            for (int i = 0; i < 16; ++i) a[swz(base + i * S)] = x[i];
        }
        __syncthreads();
    }
}

// DIT fused passes of spans between the edge block's (exclusive) and Lmax
// (inclusive): from 64, 8, 16, 32 for edge blocks 16, 2, 4, 8.  B: the edge
// block of the whole transform when a holds only sub-blocks of it (0: that
// of length n).  Ends with a barrier when it ran a pass.
template <class T>
__device__ __forceinline__ void block_dit_s_mid(Cplx<T>* a, int n, int Lmax, int B = 0) {
    if (B == 0) B = edge_block(n);
    const int L0 = B == 16 ? 64 : 4 * B;
#pragma unroll
    for (int L = L0, lL = fft_log2(L0); L <= Lmax; L <<= 4, lL += 4) {
        const int lS = lL - 2, S = 1 << lS;
        for (int g = threadIdx.x; g < (n >> 4); g += blockDim.x) {
            const int b = g & (S - 1);
            const int base = (g >> lS) * (4 * L) + b;
            Cplx<T> x[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) x[i] = a[swz(base + i * S)];
            dit16_regs(x, b, L);
#pragma unroll
            for (int i = 0; i < 16; ++i) a[swz(base + i * S)] = x[i];
        }
        __syncthreads();
    }
}
#endif
