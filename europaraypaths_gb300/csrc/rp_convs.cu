// rp_convs.cu -- the shared-memory range compression of the fast form
// (k_conv32s): per target, the chirp convolution of its trace and the
// product spectrum of u = Psour (*) Ptarg, summed over a work item's targets
// and inverse-transformed once per item (convolvePhasorChirpLinear and
// convolveComplex, radar_kernels.cu:554-649, elementary_kernels.cu:258-353).
// Its own translation unit so that it compiles beside rp_fast.cu.
#include <algorithm>

#include "rp_convs.cuh"
#include "rp_fft.cuh"
#include "rp_internal.h"

namespace rpk {

// The target's trace (the facet-range parts summed in fixed order, each
// part's row element high + low) at position k of the zero-padded 2nr input:
// zero outside the target's window [b0, b0 + Wt) and beyond nr.
__device__ __forceinline__ Cplx<float> trace_at(const C32* __restrict__ T, size_t pstride, size_t qbase, int k,
                                                int b0, int Wt, int nr) {
    Cplx<float> v{0.f, 0.f};
    const int o = k - b0;
    if (k < nr && o >= 0 && o < Wt) {
        const float4* T4 = reinterpret_cast<const float4*>(T);
        for (int p = 0; p < RP_PARTS; ++p) {
            const float4 u = T4[(size_t)p * pstride + qbase + o];
            v.x += u.x + u.z;
            v.y += u.y + u.w;
        }
    }
    return v;
}

// DIF of the zero-padded target trace into a (n values): the first fused
// pass reads its 16 inputs straight from the target's rows (only the window
// is non-zero), the rest run in place.  Ends with a barrier.
// With to_edge, the stages of the edge block are left to the caller's edge
// pass.
__device__ __forceinline__ void dif_trace(Cplx<float>* a, const C32* __restrict__ T, size_t pstride, size_t qbase,
                                          int b0, int Wt, int nr, int n, bool to_edge) {
    const int S = n >> 4;
    for (int g = threadIdx.x; g < S; g += RP_CONV_THREADS) {
        Cplx<float> x[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) x[i] = trace_at(T, pstride, qbase, g + i * S, b0, Wt, nr);
        dif16_regs(x, g, n);
#pragma unroll
        for (int i = 0; i < 16; ++i) a[swz(g + i * S)] = x[i];
    }
    __syncthreads();
    if (to_edge) block_dif_s_mid(a, n, n >> 4);
    else block_dif_s_from(a, n, n >> 4);
}

// One pass over contiguous edge blocks of B elements of src: the last DIF
// stages, then op(k0, x) (the pointwise product, the first DIT stages and the
// stores, for elements k0 .. k0 + B - 1); no barrier.
template <int B, class Op>
__device__ __forceinline__ void edge_pass(const Cplx<float>* src, int n, Op op) {
    for (int blk = threadIdx.x; blk < n / B; blk += RP_CONV_THREADS) {
        Cplx<float> x[B];
        ld_pairs<B>(src, blk * B, x);
        dif_edge<float, B>(x);
        op(blk * B, x);
    }
}

// The edge pass for the block size of length n (16, 2, 4 or 8), or eb when
// src holds sub-blocks of a longer transform.
template <class Op>
__device__ __forceinline__ void edge_pass_n(const Cplx<float>* src, int n, Op op, int eb = 0) {
    switch (eb ? eb : edge_block(n)) {
        case 16: edge_pass<16>(src, n, op); break;
        case 8: edge_pass<8>(src, n, op); break;
        case 4: edge_pass<4>(src, n, op); break;
        default: edge_pass<2>(src, n, op); break;
    }
}

// The item's sum U of the targets' product spectra.  The inverse transform
// that turns X * DIF(pad Ptarg) into u is linear, so the product spectra are
// summed over the item's targets (in target order) and transformed once per
// item.  U holds element k at swz(k), like X and W: in shared memory (mode
// 0) or in the item's partial row in global memory (modes 1 and 2).
// spec_add: one target's last DIF stages of DIF(pad Ptarg) (in W) and its
// product with X, added into U (each element by the thread that owns its
// edge block).
template <int B>
__device__ __forceinline__ void spec_add(const Cplx<float>* W, const Cplx<float>* X, Cplx<float>* U, int n) {
    for (int blk = threadIdx.x; blk < n / B; blk += RP_CONV_THREADS) {
        Cplx<float> x[B], a[B], o[B];
        ld_pairs<B>(W, blk * B, x);
        dif_edge<float, B>(x);
        ld_pairs<B>(X, blk * B, a);
        ld_pairs<B>(U, blk * B, o);
#pragma unroll
        for (int i = 0; i < B; ++i) {
            const Cplx<float> v = c_mul(a[i], x[i]);
            o[i] = Cplx<float>{o[i].x + v.x, o[i].y + v.y};
        }
        st_pairs<B>(U, blk * B, o);
    }
}

// U, scaled by sc, through the first DIT stages into W (the rest of u's
// inverse transform follows).
template <int B>
__device__ __forceinline__ void spec_to_w(Cplx<float>* W, const Cplx<float>* U, int n, float sc) {
    for (int blk = threadIdx.x; blk < n / B; blk += RP_CONV_THREADS) {
        Cplx<float> x[B];
        ld_pairs<B>(U, blk * B, x);
#pragma unroll
        for (int i = 0; i < B; ++i) x[i] = Cplx<float>{x[i].x * sc, x[i].y * sc};
        dit_edge<float, B>(x);
        st_pairs<B>(W, blk * B, x);
    }
}

// W^e = e^{-2 pi i e / n} for 0 <= e < n / 2, from the SFU at angles of
// at most pi / 2 (W^e = -i W^{e - n/4} above n / 4).
__device__ __forceinline__ Cplx<float> tw_half(int e, int n) {
    const int q = n >> 2;
    const bool hi = e >= q;
    const Cplx<float> w = tw_sfu<float>(hi ? e - q : e, 6.28318530717958647f / (float)n);
    return hi ? Cplx<float>{w.y, -w.x} : w;
}

// The first fused DIF pass of one half of a length-n transform whose input
// has its upper half zero (a zero-padded trace): half 0 transforms x, half 1
// x W^e (the span-n radix-2 stage of DIF_n is then a plain split), each as a
// length-H = n / 2 transform.  get(e) gives x[e], e < H.  Into a (swizzled).
template <class Get>
__device__ __forceinline__ void half_first_pass(Cplx<float>* a, int H, int h, Get get) {
    const int SH = H >> 4;
    for (int g = threadIdx.x; g < SH; g += RP_CONV_THREADS) {
        Cplx<float> x[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int e = g + i * SH;
            const Cplx<float> v = get(e);
            x[i] = h ? c_mul(v, tw_half(e, 2 * H)) : v;
        }
        dif16_regs(x, g, H);
#pragma unroll
        for (int i = 0; i < 16; ++i) a[swz(g + i * SH)] = x[i];
    }
}

// The last fused DIT pass of a length-H transform: natural-order outputs,
// unscaled, into dst (swizzled; dst may be a).
__device__ __forceinline__ void half_last_dit(const Cplx<float>* a, Cplx<float>* dst, int H) {
    const int SH = H >> 4;
    for (int g = threadIdx.x; g < SH; g += RP_CONV_THREADS) {
        Cplx<float> x[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) x[i] = a[swz(g + i * SH)];
        dit16_regs(x, g, H >> 2);
#pragma unroll
        for (int i = 0; i < 16; ++i) dst[swz(g + i * SH)] = x[i];
    }
}

// One work item of k_conv32s (below).  NC: the transform length 2nr
// as a compile-time constant for the common lengths (0: the job's, at run
// time), so the passes' strides, twiddle steps and loop trip counts fold.
template <int MODE, bool SPEC, int NC>
__device__ __forceinline__ void conv_item(const ConvArgs& A, unsigned int item, Cplx<float>* const sbase,
                                          Cplx<float>* const gbase) {
    const int tid = threadIdx.x;
    const int nr = A.nr, n2 = NC ? NC : A.n2, N = A.N;
    const int S = n2 >> 4;                  // groups of the outer fused passes
    // X: DIF(pad T) (and DIF(pad T2) in specular mode); W: the working transform
    Cplx<float>* const X = (MODE == 2) ? gbase : (MODE == 1 ? gbase : sbase);
    Cplx<float>* const W = (MODE == 0) ? sbase + n2 : (MODE == 1 ? sbase : gbase + n2);
    // the job's arguments in registers (the loops below store to shared
    // memory, which would otherwise force re-reads of A)
    const Cplx<float>* __restrict__ C2s = A.C2s;
    const C32* __restrict__ T = A.T;
    const C32* __restrict__ T2 = A.T2;
    const int Wt = A.Wt, nsplit = A.nsplit;
    const int64_t tstride = A.tstride;
    const size_t pstride = (size_t)A.nb * tstride * Wt;
    const float sig_scale = A.sig_scale;
    const int* __restrict__ bt0 = A.bt0;
    C32* __restrict__ part = A.part;
    const int s = item / nsplit;
    const int sp = item % nsplit;
    const int nq = A.ntl[s];
    const int q0 = sp * RP_CONV_SPLIT;
    if (q0 >= nq) return;
    const int q1 = min(q0 + RP_CONV_SPLIT, nq);
    C32* const out = part + ((size_t)s * nsplit + sp) * n2;
    // U: the summed product spectra (spec_add); mode 0 in shared memory
    // after X and W, else the item's partial row, which then receives u
    Cplx<float>* const U = (MODE == 0) ? sbase + 2 * n2 : reinterpret_cast<Cplx<float>*>(out);
    for (int j = tid; j < n2; j += RP_CONV_THREADS) U[j] = Cplx<float>{0.f, 0.f};
    const float inv = 1.f / (float)n2;
    const float sc = sig_scale / (float)n2;
    const int EB = edge_block(n2);
    const int SB = n2 >> 4;                 // mode 2: sub-block of the inner stages
    const bool blocked = MODE == 2 && SB <= RP_CONV_CHUNK;
    // mode 2 at 2nr = 2 RP_CONV_CHUNK runs by halves (below); its spectra
    // (the chirp's C2s included) are in the halves' order
    constexpr bool HALVES = MODE == 2 && NC == 2 * RP_CONV_CHUNK;
    constexpr int HH = RP_CONV_CHUNK;       // the half length
    const int EBH = edge_block(HH);
    for (int q = q0; q < q1; ++q) {
        const int b0 = bt0[(size_t)s * tstride + q];
        const size_t qbase = ((size_t)s * tstride + q) * Wt;
        if constexpr (HALVES) {
            // ---- mode 2 at 2nr = 2 RP_CONV_CHUNK, by halves.  The input
            // of every forward transform is a zero-padded trace, so DIF_n's
            // first (span-n radix-2) stage splits it into x and x W^e, two
            // independent length-H transforms run whole in shared memory;
            // the spectra live in that split order ([DIF_H(x); DIF_H(x
            // W^e)], the chirp's C2s included).  The inverse joins the two
            // halves' DIT_H outputs a, b as y[e] = a[e] + W^-e b[e], y[e +
            // H] = a[e] - W^-e b[e]; Ptarg needs y[nr/2 .. 3nr/2) only.
            // Global slot: X (halves at 0 and H), then Wa (H values).
            Cplx<float>* const Wa = gbase + n2;
            const C32* __restrict__ Tr = T;
            for (int h = 0; h < 2; ++h) {
                half_first_pass(sbase, HH, h, [&](int e) { return trace_at(Tr, pstride, qbase, e, b0, Wt, nr); });
                __syncthreads();
                block_dif_s_mid(sbase, HH, HH >> 4);
                Cplx<float>* const Xh = X + h * HH;
                const Cplx<float>* const Ch = C2s + h * HH;
                edge_pass_n(sbase, HH, [&](int k0, auto& x) {
                    constexpr int B = sizeof(x) / sizeof(x[0]);
                    st_pairs<B>(Xh, k0, x);
#pragma unroll
                    for (int i = 0; i < B; i += 2) {
                        const float4 c = *reinterpret_cast<const float4*>(Ch + k0 + i);
                        x[i] = c_mul(x[i], Cplx<float>{c.x, c.y});
                        x[i + 1] = c_mul(x[i + 1], Cplx<float>{c.z, c.w});
                    }
                    dit_edge<float, B>(x);
                    st_pairs<B>(sbase, k0, x);
                });
                __syncthreads();
                block_dit_s_mid(sbase, HH, HH >> 4);
                half_last_dit(sbase, h == 0 ? Wa : sbase, HH);     // a to the slot, b in place
                __syncthreads();
            }
            // Ptarg[k] = y[k + nr/2] / n: Ptarg[e] = a[e+Q] + W^-(e+Q) b[e+Q],
            // Ptarg[e+Q] = a[e] - W^-e b[e] (Q = H / 2 = 8 SH), to Wa, and
            // in the same registers the first DIF pass of half 0 of
            // DIF(pad Ptarg): group g's elements g + i SH are the pairs' e
            // (i < 8) and e + Q (i >= 8), e = g + i SH
            {
                constexpr int SH = HH >> 4, Q = HH >> 1;
                for (int g = tid; g < SH; g += RP_CONV_THREADS) {
                    Cplx<float> x[16];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int e = g + i * SH, e1 = e + Q;
                        const Cplx<float> a0 = Wa[swz(e)], a1 = Wa[swz(e1)];
                        const Cplx<float> t0 = c_mulc(sbase[swz(e)], tw_half(e, n2));
                        const Cplx<float> t1 = c_mulc(sbase[swz(e1)], tw_half(e1, n2));
                        x[i] = Cplx<float>{(a1.x + t1.x) * inv, (a1.y + t1.y) * inv};
                        x[i + 8] = Cplx<float>{(a0.x - t0.x) * inv, (a0.y - t0.y) * inv};
                    }
#pragma unroll
                    for (int i = 0; i < 16; ++i) Wa[swz(g + i * SH)] = x[i];
                    dif16_regs(x, g, HH);
#pragma unroll
                    for (int i = 0; i < 16; ++i) sbase[swz(g + i * SH)] = x[i];
                }
                __syncthreads();
            }
            if constexpr (SPEC) {
                // Psour = s T2: its transform's halves replace X
                const C32* __restrict__ T2r = T2;
                for (int h = 0; h < 2; ++h) {
                    half_first_pass(sbase, HH, h,
                                    [&](int e) { return trace_at(T2r, pstride, qbase, e, b0, Wt, nr); });
                    __syncthreads();
                    block_dif_s_from(sbase, HH, HH >> 4);
                    for (int k = tid; k < HH; k += RP_CONV_THREADS) X[h * HH + k] = sbase[k];
                    __syncthreads();
                }
            }
            // DIF(pad Ptarg) by halves, each's product with X added into U
            for (int h = 0; h < 2; ++h) {
                if (SPEC || h == 1) {
                    half_first_pass(sbase, HH, h, [&](int e) { return Wa[swz(e)]; });
                    __syncthreads();
                }
                block_dif_s_mid(sbase, HH, HH >> 4);
                switch (EBH) {
                    case 16: spec_add<16>(sbase, X + h * HH, U + h * HH, HH); break;
                    case 8: spec_add<8>(sbase, X + h * HH, U + h * HH, HH); break;
                    case 4: spec_add<4>(sbase, X + h * HH, U + h * HH, HH); break;
                    default: spec_add<2>(sbase, X + h * HH, U + h * HH, HH); break;
                }
                __syncthreads();
            }
            continue;
        }
        if (blocked) {
            // ---- mode 2 by sub-blocks: the stages of spans <= n / 16
            // act within contiguous sub-blocks of SB = n / 16 elements,
            // so they run in shared memory, RP_CONV_CHUNK elements at a
            // time; only the outer fused passes (spans n, n / 4) go to
            // the global slot.  P1: the first DIF pass from the rows
            for (int g = tid; g < S; g += RP_CONV_THREADS) {
                Cplx<float> x[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) x[i] = trace_at(T, pstride, qbase, g + i * S, b0, Wt, nr);
                dif16_regs(x, g, n2);
#pragma unroll
                for (int i = 0; i < 16; ++i) W[swz(g + i * S)] = x[i];
            }
            __syncthreads();
            // P2, per chunk: the rest of DIF(pad T), X stored, the
            // product with C2, the DIT stages of spans <= SB
            for (int c0 = 0; c0 < n2; c0 += RP_CONV_CHUNK) {
                for (int k = tid; k < RP_CONV_CHUNK; k += RP_CONV_THREADS) sbase[k] = W[c0 + k];
                __syncthreads();
                block_dif_s_mid(sbase, RP_CONV_CHUNK, SB);
                Cplx<float>* const Xc = X + c0;
                const Cplx<float>* const Cc = C2s + c0;
                edge_pass_n(sbase, RP_CONV_CHUNK, [&](int k0, auto& x) {
                    constexpr int B = sizeof(x) / sizeof(x[0]);
                    st_pairs<B>(Xc, k0, x);
#pragma unroll
                    for (int i = 0; i < B; i += 2) {
                        const float4 c = *reinterpret_cast<const float4*>(Cc + k0 + i);
                        x[i] = c_mul(x[i], Cplx<float>{c.x, c.y});
                        x[i + 1] = c_mul(x[i + 1], Cplx<float>{c.z, c.w});
                    }
                    dit_edge<float, B>(x);
                    st_pairs<B>(sbase, k0, x);
                }, EB);
                __syncthreads();
                block_dit_s_mid(sbase, RP_CONV_CHUNK, SB >> 2, EB);
                for (int k = tid; k < RP_CONV_CHUNK; k += RP_CONV_THREADS) W[c0 + k] = sbase[k];
                __syncthreads();
            }
            // P3: the last DIT pass, the shift, the first DIF pass (global)
            for (int g = tid; g < S; g += RP_CONV_THREADS) {
                Cplx<float> x[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) x[i] = W[swz(g + i * S)];
                dit16_regs(x, g, n2 >> 2);
#pragma unroll
                for (int i = 0; i < 8; ++i) x[i] = Cplx<float>{x[i + 4].x * inv, x[i + 4].y * inv};
#pragma unroll
                for (int i = 8; i < 16; ++i) x[i] = Cplx<float>{0.f, 0.f};
                dif16_regs(x, g, n2);
#pragma unroll
                for (int i = 0; i < 16; ++i) W[swz(g + i * S)] = x[i];
            }
            __syncthreads();
            if constexpr (SPEC) dif_trace(X, T2, pstride, qbase, b0, Wt, nr, n2, false);
            // P4, per chunk: the rest of DIF(pad Ptarg) and the product
            // with X, added into U
            for (int c0 = 0; c0 < n2; c0 += RP_CONV_CHUNK) {
                for (int k = tid; k < RP_CONV_CHUNK; k += RP_CONV_THREADS) sbase[k] = W[c0 + k];
                __syncthreads();
                block_dif_s_mid(sbase, RP_CONV_CHUNK, SB);
                switch (EB) {
                    case 16: spec_add<16>(sbase, X + c0, U + c0, RP_CONV_CHUNK); break;
                    case 8: spec_add<8>(sbase, X + c0, U + c0, RP_CONV_CHUNK); break;
                    case 4: spec_add<4>(sbase, X + c0, U + c0, RP_CONV_CHUNK); break;
                    default: spec_add<2>(sbase, X + c0, U + c0, RP_CONV_CHUNK); break;
                }
                __syncthreads();
            }
            continue;
        }
        // ---- X = DIF(pad T) up to its edge block (mode 1: in W's
        // shared memory), then one edge pass: the last DIF stages, X
        // stored (mode 1: parked in the slot), W = X * C2 and the first
        // DIT stages of Ptarg's transform
        Cplx<float>* const D1 = (MODE == 1) ? W : X;
        dif_trace(D1, T, pstride, qbase, b0, Wt, nr, n2, true);
        edge_pass_n(D1, n2, [&](int k0, auto& x) {
            constexpr int B = sizeof(x) / sizeof(x[0]);
            st_pairs<B>(X, k0, x);
#pragma unroll
            for (int i = 0; i < B; i += 2) {
                const float4 c = *reinterpret_cast<const float4*>(C2s + k0 + i);
                x[i] = c_mul(x[i], Cplx<float>{c.x, c.y});
                x[i + 1] = c_mul(x[i + 1], Cplx<float>{c.z, c.w});
            }
            dit_edge<float, B>(x);
            st_pairs<B>(W, k0, x);
        });
        __syncthreads();
        // ---- Ptarg: the DIT passes up to span n/16, then the last fused
        // pass, the shift by nr/2 with the 1/2nr scale and zero padding,
        // and the first DIF pass of DIF(pad Ptarg), in registers
        block_dit_s_mid(W, n2, n2 >> 4);
        for (int g = tid; g < S; g += RP_CONV_THREADS) {
            Cplx<float> x[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) x[i] = W[swz(g + i * S)];
            dit16_regs(x, g, n2 >> 2);
#pragma unroll
            for (int i = 0; i < 8; ++i) x[i] = Cplx<float>{x[i + 4].x * inv, x[i + 4].y * inv};
#pragma unroll
            for (int i = 8; i < 16; ++i) x[i] = Cplx<float>{0.f, 0.f};
            dif16_regs(x, g, n2);
#pragma unroll
            for (int i = 0; i < 16; ++i) W[swz(g + i * S)] = x[i];
        }
        __syncthreads();
        // specular mode: Psour = s T2, the outbound leg's own trace, whose
        // transform replaces X (X's DIF(pad T) is no longer needed)
        if constexpr (SPEC) dif_trace(X, T2, pstride, qbase, b0, Wt, nr, n2, false);
        block_dif_s_mid(W, n2, n2 >> 4);
        // ---- DIF(pad Ptarg)'s last stages and the spectra's product,
        // added into the item's sum
        switch (EB) {
            case 16: spec_add<16>(W, X, U, n2); break;
            case 8: spec_add<8>(W, X, U, n2); break;
            case 4: spec_add<4>(W, X, U, n2); break;
            default: spec_add<2>(W, X, U, n2); break;
        }
        __syncthreads();    // X and W are read above; the next target overwrites them
    }
    // ---- the item's u = s / 2nr DIT(sum of the product spectra); the
    // last fused pass writes the N values in natural order
    if constexpr (HALVES) {
        // u = s / 2nr DIT(U) by halves: DIT_H of each half of U, then the
        // join y[e] = a[e] + W^-e b[e], y[e + H] = a[e] - W^-e b[e] into
        // the item's row (which held U: both halves are read before it is
        // written)
        Cplx<float>* const Wa = gbase + n2;
        for (int h = 0; h < 2; ++h) {
            for (int k = tid; k < HH; k += RP_CONV_THREADS) {
                const Cplx<float> o = U[h * HH + k];
                sbase[k] = Cplx<float>{o.x * sc, o.y * sc};
            }
            __syncthreads();
            block_dit_s(sbase, HH);
            if (h == 0) {
                for (int k = tid; k < HH; k += RP_CONV_THREADS) Wa[k] = sbase[k];
                __syncthreads();
            }
        }
        for (int e = tid; e < HH; e += RP_CONV_THREADS) {
            const Cplx<float> a = Wa[swz(e)];
            const Cplx<float> t = c_mulc(sbase[swz(e)], tw_half(e, n2));
            out[e] = C32{a.x + t.x, a.y + t.y};
            if (e + HH < N) out[e + HH] = C32{a.x - t.x, a.y - t.y};
        }
        return;
    }
    if (blocked) {
        for (int c0 = 0; c0 < n2; c0 += RP_CONV_CHUNK) {
            switch (EB) {
                case 16: spec_to_w<16>(sbase, U + c0, RP_CONV_CHUNK, sc); break;
                case 8: spec_to_w<8>(sbase, U + c0, RP_CONV_CHUNK, sc); break;
                case 4: spec_to_w<4>(sbase, U + c0, RP_CONV_CHUNK, sc); break;
                default: spec_to_w<2>(sbase, U + c0, RP_CONV_CHUNK, sc); break;
            }
            __syncthreads();
            block_dit_s_mid(sbase, RP_CONV_CHUNK, SB >> 2, EB);
            for (int k = tid; k < RP_CONV_CHUNK; k += RP_CONV_THREADS) W[c0 + k] = sbase[k];
            __syncthreads();
        }
    } else {
        switch (EB) {
            case 16: spec_to_w<16>(W, U, n2, sc); break;
            case 8: spec_to_w<8>(W, U, n2, sc); break;
            case 4: spec_to_w<4>(W, U, n2, sc); break;
            default: spec_to_w<2>(W, U, n2, sc); break;
        }
        __syncthreads();
        block_dit_s_mid(W, n2, n2 >> 4);
    }
    for (int g = tid; g < S; g += RP_CONV_THREADS) {
        Cplx<float> x[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) x[i] = W[swz(g + i * S)];
        dit16_regs(x, g, n2 >> 2);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int j = g + i * S;
            if (j < N) out[j] = C32{x[i].x, x[i].y};
        }
    }
}

// Shared-memory range compression (nr a power of two >= 16).  One work item =
// RP_CONV_SPLIT consecutive targets of one trace; their contributions are
// summed in target order and written as one partial trace.  Per target (n =
// 2nr values in X and W):
//   X = DIF(pad T)                         T = sum of the facet-range parts
//   W = DIT(X * C2)[nr/2 ..] / 2nr         Ptarg (convolvePhasorChirpLinear)
//   U += X * DIF(pad Ptarg)                the product spectrum of u = Psour (*)
//                                          Ptarg, Psour = s T (specular: X =
//                                          DIF(pad T2) first); length N =
//                                          2nr - 1, so the N-point circular
//                                          product has no wrap
// and per item u = DIT(U) * s / 2nr: the inverse transform is linear, so the
// targets' product spectra are summed and transformed once (3 transforms a
// target instead of 4).  The rest of the chain (cropSpectrum, the inverse
// N-point DFT, takeEveryOtherComplex) is linear in u and the same for every
// target, so it runs once per trace on the sum (k_trace_m32).  The
// transforms are the in-place stages of rp_fft.cuh with the elements at
// swizzled positions, and four pass boundaries are crossed in registers
// instead of shared memory:
//  * the first DIF pass of X reads the target's rows directly;
//  * the last DIF stages of X, the product with the chirp spectrum and the
//    first DIT stages of Ptarg's transform act on the same contiguous edge
//    blocks (rp_fft.cuh: edge_block), so they run as one edge pass;
//  * Ptarg is a shift by nr/2 = 4 S of the first transform's natural-order
//    output, S = n / 16, and the first DIF pass of the second transform reads
//    elements g + i S (i < 8 non-zero) -- exactly the registers x[i + 4] that
//    the last DIT pass of the first transform leaves in the same thread -- so
//    the two passes and the shift run back to back in registers;
//  * the last DIF stages of DIF(pad Ptarg) and the spectra's product run in
//    the edge pass that adds into U (spec_add).
// Persistent over the items of one or more batches (job j owns items
// [start[j], start[j + 1])); twiddles come from the SFU.  MODE 0: X, W and U
// in shared memory (nr <= 4096; 192 KiB at nr = 4096).  MODE 1 (nr = 8192): every
// transform in one n-value buffer of shared memory; X waits in this block's
// slot of the global scratch between its two uses.  MODE 2: X and W in the
// slot (nr >= 16384).  Modes 1 and 2 keep U in the item's partial row in
// global memory (same element, same target order as mode 0, so every mode
// gives the same sums), which then receives u.
template <int MODE, bool SPEC, int NC>
__global__ void __launch_bounds__(RP_CONV_THREADS, 1)
k_conv32s(const ConvArgs* __restrict__ jobs, const unsigned int* __restrict__ start, int njobs,
          unsigned int* work, Cplx<float>* __restrict__ gscr, size_t gslot) {
    extern __shared__ __align__(16) unsigned char csm[];
    Cplx<float>* const sbase = reinterpret_cast<Cplx<float>*>(csm);
    Cplx<float>* const gbase = gscr + (size_t)blockIdx.x * gslot;
    __shared__ unsigned int s_item;
    __shared__ int s_job;
    __shared__ ConvArgs A;                  // the current item's job (off the FFT hot path)
    const int tid = threadIdx.x;
    const unsigned int total = start[njobs];
    int curJ = -1;
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
        __syncthreads();        // every thread is done with the previous item's A
        const unsigned int item0 = s_item;
        const int jb = s_job;
        if (tid == 0 && item0 < total && jb != curJ) A = jobs[jb];
        __syncthreads();
        if (item0 >= total) break;
        curJ = jb;
        conv_item<MODE, SPEC, NC>(A, item0 - start[jb], sbase, gbase);
    }
}

// Transform lengths 2nr with a kernel of their own (the lengths of the
// measured workloads); a job table holds one length class of one mode.
int conv_length_class(int mode, int n2) {
    if (mode == 0) return (n2 == 8192 || n2 == 4096) ? n2 : 0;
    if (mode == 1) return n2 == 16384 ? n2 : 0;
    return n2 == 32768 ? n2 : 0;
}

template <int MODE, bool SPEC, int NC>
int launch_conv_k(const ConvArgs* d_jobs, const unsigned int* d_start, int njobs, size_t csm, int sms, int slots,
                  unsigned int items, unsigned int* work, C32* gscr, size_t gslot, cudaStream_t st) {
    auto kern = k_conv32s<MODE, SPEC, NC>;
    if (int rc = rp_allow_dyn_smem((const void*)kern, csm)) return rc;
    int occ = 0;
    RP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, RP_CONV_THREADS, csm));
    int64_t gmax = (int64_t)std::max(occ, 1) * sms;
    if (MODE != 0) gmax = std::min<int64_t>(gmax, slots);      // one scratch slot per block
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(gmax, items));
    kern<<<grid, RP_CONV_THREADS, csm, st>>>(d_jobs, d_start, njobs, work, reinterpret_cast<Cplx<float>*>(gscr),
                                             gslot);
    RP_CUDA(cudaGetLastError());
    RP_LAUNCHED();
    return RP_OK;
}

template <bool SPEC>
int launch_conv32s_t(const ConvArgs* d_jobs, const unsigned int* d_start, int njobs, int mode, int nc,
                     size_t csm, int sms, int slots, unsigned int items, unsigned int* work, C32* gscr,
                     size_t gslot, cudaStream_t st) {
#define RP_CONV_ARGS d_jobs, d_start, njobs, csm, sms, slots, items, work, gscr, gslot, st
    if (mode == 1) {
        if (nc == 16384) return launch_conv_k<1, SPEC, 16384>(RP_CONV_ARGS);
        return launch_conv_k<1, SPEC, 0>(RP_CONV_ARGS);
    }
    if (mode == 2) {
        if (nc == 32768) return launch_conv_k<2, SPEC, 32768>(RP_CONV_ARGS);
        return launch_conv_k<2, SPEC, 0>(RP_CONV_ARGS);
    }
    if (nc == 8192) return launch_conv_k<0, SPEC, 8192>(RP_CONV_ARGS);
    if (nc == 4096) return launch_conv_k<0, SPEC, 4096>(RP_CONV_ARGS);
    return launch_conv_k<0, SPEC, 0>(RP_CONV_ARGS);
#undef RP_CONV_ARGS
}

int launch_conv32s(const ConvArgs* d_jobs, const unsigned int* d_start, int njobs, int mode, int nc,
                   size_t csm, int sms, int slots, unsigned int items, unsigned int* work, C32* gscr,
                   size_t gslot, bool spec, cudaStream_t st) {
    return spec ? launch_conv32s_t<true>(d_jobs, d_start, njobs, mode, nc, csm, sms, slots, items, work, gscr,
                                         gslot, st)
                : launch_conv32s_t<false>(d_jobs, d_start, njobs, mode, nc, csm, sms, slots, items, work, gscr,
                                          gslot, st);
}

}  // namespace rpk
