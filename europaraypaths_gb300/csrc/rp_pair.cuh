// rp_pair.cuh -- the pair stage of the fast form, shared by the single-batch
// kernel (rp_fast.cu) and the multi-job kernel (rp_multi.cu): the per-facet
// record, the TMA bulk staging helpers, the FP32 split-precision evaluation of
// one (facet, target) pair (compTargetRays, compRefrEnergyIn,
// accumulateTarget: geometry_kernels.cu:272-350, 520-554,
// radar_kernels.cu:767-830), the deterministic window binning and the body
// of one work item.
//
// The two kernels live in separate translation units: compiled together, the
// multi-job kernel's call sites of the out-of-line helpers changed the code
// generated for the single-batch kernel (8% slower on the large scene).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "rp_math.cuh"

#define RP_CHUNK 256          // facets per chunk (one record tile)
#define RP_PAIR_THREADS 256   // targets per pair-kernel block
#define RP_WIN 16             // bins in a thread's per-chunk window
#define RP_PARTS 4            // facet-range splits per (trace, target block)
#define RP_SPIN_LIMIT (1 << 22)

namespace rpk {

using C32 = Cx<float>;

struct __align__(16) FacetRec {
    float4 a;   // dx, dy, dz (facet - chunk centre), |d|^2
    float4 b;   // nx, ny, nz, xI = (Itd - rst) / dr
    float4 c;   // ux, uy, uz, tauI = frac(Itd / lam)
    float4 d;   // vx, vy, vz, K = amplitude factor
};

struct __align__(16) ChunkMeta {
    double cx, cy, cz;     // chunk centre
    float R;               // max |facet - centre|
    float xmin, xmax;      // range of (Itd - rst)/dr
    int n;                 // facets in the chunk
    double bbmin[3], bbmax[3];
};

// ------------------------------------------------------------ TMA bulk --
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void tma_bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Bounded wait on an mbarrier phase; returns false if the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase) {
    for (int it = 0; it < RP_SPIN_LIMIT; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

// ----------------------------------------------------------- pair kernel --
struct PairArgs {
    const FacetRec* rec;
    const ChunkMeta* meta;
    int64_t rstride, mstride;
    const int* nill;
    const int* ntl;
    const int* tlist;
    int64_t tstride;
    const double* TG;
    int64_t nt;
    const double* PR;   // prisms (alpha, box) FP64 SoA
    int64_t np;
    const int* bt0;
    C32* T;             // [RP_PARTS][nb][tstride][Wt]
    int Wt;
    int nb;
    int tblocks;        // target blocks per trace
    unsigned int* work; // work counter
    unsigned int* err;  // error flags: [0] window overflow, [1] wait timeout
    // constants
    float nr_f;
    int nr;
    int nr1;            // nr - 1: both split bins are inside the trace when b < nr - 1
    float kb;           // n / dr
    float kt;           // n / lam
    float pik;          // pi * (pi_F * fs / lam): sinc arguments in radians
    float pik2;         // pik^2
    float sc[8];        // sinc polynomial coefficients in t = a^2 (sinc_poly)
    float ealpha;       // -2 alpha2 log2(e)
    float eks;          // -2 ks^2 log2(e)
    double nidx, inv_dr, inv_lam;   // inv_lam: turns per metre, pi_F / (pi lam)
    int lossless;
};

// A job of the multi-job pair kernel: a batch's arguments and its sinc
// polynomial degree (0: special-function unit).
struct PairJob {
    PairArgs a;
    int deg;
};

// Per-(chunk, target) anchors of the split-precision evaluation.
struct Anchor {
    float Dx, Dy, Dz;     // target - chunk centre (FP32 of an FP64 difference)
    float T0, T0sq;       // |target - chunk centre| (FP64 -> FP32)
    float tau0;           // frac(n T0 turn): phase of the anchor in turns
    float xbase;          // n T0 / dr - blo (bins, relative to the window start)
    float tnx, tny, tnz;  // target normal
    float eaT0;           // ealpha T0: the attenuation exponent at the anchor
};

// Hardware approximations (PTX rsqrt/rcp/ex2 .approx.ftz): single
// special-function-unit instructions, relative error ~2^-22.
__device__ __forceinline__ float rsqrt_a(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_a(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float ex2_a(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// sin(a)/a as a degree-D polynomial in t = a^2 (coefficients fitted per
// scene on [0, amax^2], see sinc_poly), Horner form.
template <int D>
__device__ __forceinline__ float sinc_poly_eval(const float* c, float t) {
    float s = c[D];
#pragma unroll
    for (int k = D - 1; k >= 0; --k) s = fmaf(s, t, c[k]);
    return s;
}

// One (facet, target) evaluation of the target leg (compTargetRays,
// compRefrEnergyIn, accumulateTarget; geometry_kernels.cu:272-350, 520-554,
// radar_kernels.cu:767-830).  Returns the phasor and x - blo, the bin
// coordinate relative to the window start.
//
// The two directivities facet_G(Tth, Tph) and facet_G(TargetTh, Tph)
// (radar_kernels.cu:658-677) need sinc(pik/pi * sin(th) cos(ph)) and
// sinc(pik/pi * sin(th) sin(ph)), sinc(x) = sin(pi x)/(pi x).  With
// cos(Tph) = xv / sqrt(h2), sin(Tph) = yu / sqrt(h2) and sin^2(th) = 1 - c^2,
// the squared sinc arguments are pik^2 (1 - c^2) xv^2 / h2 etc. (atan2(0, 0)
// = 0 gives xv^2/h2 = 1, yu^2/h2 = 0).  NT > 0 evaluates sin(a)/a as a
// polynomial in a^2 (no special-function unit); NT == 0 uses sin(a)/a with
// one shared reciprocal, 1 for |a| < pi 1e-6 (elementary_kernels.cu:50-53).
// RED: reduce the phase to [-1/2, 1/2] turns before the special-function
// sine and cosine; the fast path skips it when the chunk keeps |tau| below
// 42 turns (sin/cos.approx hold their accuracy over +-100 pi radians).
template <int NT, bool RED = true>
__device__ __forceinline__ void pair_eval(const FacetRec& r, const Anchor& an, const PairArgs& A,
                                          float& xr, float& vre, float& vim) {
    const float dd = fmaf(an.Dx, r.a.x, fmaf(an.Dy, r.a.y, an.Dz * r.a.z));
    const float qd = fmaf(-2.f, dd, r.a.w);             // Ttd^2 - T0^2
    const float d2 = an.T0sq + qd;
    const float rinv = rsqrt_a(d2);
    const float dT = qd * rcp_a(fmaf(d2, rinv, an.T0));  // Ttd - T0 without cancellation
    float S, cT2;
    if (NT > 0) {
        // The polynomial sinc needs only ratios of the direction's dot
        // products, so the direction e = target - facet is not normalised:
        // cos^2(Tth) = (e.n)^2 / |e|^2, 1 - cos^2 per angle, and the squared
        // in-plane split xx = pik^2 (e.v)^2 / ((e.u)^2 + (e.v)^2), yy =
        // pik^2 - xx (atan2(0, 0) = 0 gives xx = pik^2, yy = 0).  1 - c^2 may
        // round a hair below 0 for |c| ~ 1: harmless in the polynomial.
        const float ex = an.Dx - r.a.x, ey = an.Dy - r.a.y, ez = an.Dz - r.a.z;
        const float pb = fmaf(ex, r.b.x, fmaf(ey, r.b.y, ez * r.b.z));
        const float pt = fmaf(ex, an.tnx, fmaf(ey, an.tny, ez * an.tnz));
        const float pc = fmaf(ex, r.c.x, fmaf(ey, r.c.y, ez * r.c.z));
        const float pd = fmaf(ex, r.d.x, fmaf(ey, r.d.y, ez * r.d.z));
        const float inv_d2 = rcp_a(d2);
        const float pb2 = pb * pb;
        cT2 = pb2 * inv_d2;
        const float aT = 1.f - cT2;
        const float aD = fmaf(-pt * pt, inv_d2, 1.f);
        const float X = pd * pd;
        const float h2 = fmaf(pc, pc, X);
        const bool hz = !(h2 > 0.f);
        const float k2 = A.pik2 * rcp_a(h2);
        const float xx = hz ? A.pik2 : k2 * X;
        const float yy = A.pik2 - xx;
        S = sinc_poly_eval<(NT > 0 ? NT : 1)>(A.sc, aT * xx) * sinc_poly_eval<(NT > 0 ? NT : 1)>(A.sc, aT * yy) *
            sinc_poly_eval<(NT > 0 ? NT : 1)>(A.sc, aD * xx) * sinc_poly_eval<(NT > 0 ? NT : 1)>(A.sc, aD * yy);
    } else {
        const float jx = (an.Dx - r.a.x) * rinv;
        const float jy = (an.Dy - r.a.y) * rinv;
        const float jz = (an.Dz - r.a.z) * rinv;
        float cT = -fmaf(jx, r.b.x, fmaf(jy, r.b.y, jz * r.b.z));
        float cD = -fmaf(jx, an.tnx, fmaf(jy, an.tny, jz * an.tnz));
        const float yu = fmaf(jx, r.c.x, fmaf(jy, r.c.y, jz * r.c.z));
        const float xv = fmaf(jx, r.d.x, fmaf(jy, r.d.y, jz * r.d.z));
        const float h2 = fmaf(yu, yu, xv * xv);
        cT = fminf(1.f, fmaxf(-1.f, cT));
        cD = fminf(1.f, fmaxf(-1.f, cD));
        cT2 = cT * cT;
        const float aT = fmaf(-cT, cT, 1.f);
        const float aD = fmaf(-cD, cD, 1.f);
        const bool hz = !(h2 > 0.f);
        const float pT = aT * h2, pD = aD * h2;
        const float gT = (pT > 0.f) ? aT * rsqrtf(pT) : 0.f;
        const float gD = (pD > 0.f) ? aD * rsqrtf(pD) : 0.f;
        const float a1 = A.pik * (hz ? sqrtf(aT) : gT * xv);
        const float a2 = A.pik * (hz ? 0.f : gT * yu);
        const float a3 = A.pik * (hz ? sqrtf(aD) : gD * xv);
        const float a4 = A.pik * (hz ? 0.f : gD * yu);
        const float eps = 3.14159265e-6f;
        const bool z1 = fabsf(a1) < eps, z2 = fabsf(a2) < eps, z3 = fabsf(a3) < eps, z4 = fabsf(a4) < eps;
        const float num = (z1 ? 1.f : __sinf(a1)) * (z2 ? 1.f : __sinf(a2)) * (z3 ? 1.f : __sinf(a3)) *
                          (z4 ? 1.f : __sinf(a4));
        const float den = (z1 ? 1.f : a1) * (z2 ? 1.f : a2) * (z3 ? 1.f : a3) * (z4 ? 1.f : a4);
        S = __fdividef(num, den);
    }
    // attenuation and roughness (zero constants when lossless); ealpha Ttd
    // = ealpha T0 + ealpha (Ttd - T0)
    const float e2 = fmaf(A.eks, cT2, fmaf(A.ealpha, dT, an.eaT0));
    const float amp = r.d.w * fabsf(S) * rinv * ex2_a(e2);
    float tau = (r.c.w + an.tau0) + A.kt * dT;
    if (RED) tau -= rintf(tau);
    float sn, cs;
    __sincosf(-6.28318530717958647f * tau, &sn, &cs);
    vre = amp * cs;
    vim = amp * sn;
    xr = r.b.w + an.xbase + A.kb * dT;
}

// Attenuation-prism factor for one pair (compTargetRays, geometry_kernels.cu:
// 317-342): exp2 of the change of the exponent from alpha2 * Ttd to
// sum(alpha_p d_p) + alpha2 (Ttd - sum d_p).
static __device__ __noinline__ float prism_factor(float4 ra, double cx, double cy, double cz, float Dx,
                                           float Dy, float Dz, float T0sq, const double* PR,
                                           int64_t np, float ealpha) {
    const float dd = fmaf(Dx, ra.x, fmaf(Dy, ra.y, Dz * ra.z));
    const float d2 = T0sq + fmaf(-2.f, dd, ra.w);
    const float rinv = rsqrtf(d2);
    const float Ttd = d2 * rinv;
    const double fx = cx + ra.x, fy = cy + ra.y, fz = cz + ra.z;
    const double jx = (Dx - ra.x) * rinv, jy = (Dy - ra.y) * rinv, jz = (Dz - ra.z) * rinv;
    double tot = 0.0, ex = 0.0;
    for (int64_t p = 0; p < np; ++p) {
        double box[6] = {PR[np + p], PR[2 * np + p], PR[3 * np + p],
                         PR[4 * np + p], PR[5 * np + p], PR[6 * np + p]};
        double ad = d_prism_dist(fx, fy, fz, jx, jy, jz, box, Ttd);
        tot += ad;
        ex += PR[p] * ad;
    }
    // ealpha = -2 alpha2 log2(e): replace alpha2 * tot by the prisms' sum
    return exp2f(-ealpha * (float)tot - 2.f * 1.44269504f * (float)ex);
}

// Add one phasor into the thread's window (or, outside it, directly into the
// thread's own trace row).  Bin and weight follow the reference's two-bin
// split: b = (short)x (truncation), w = x - b (radar_kernels.cu:736-760).
// floor(xr) comes from rounding xr - 1/2 with the 1.5 * 2^23 magic number
// (an exact half rounds either way; the split is continuous there, so both
// give the same contributions); x in (-1, 0) is truncated to bin 0 as the
// reference does.
static __device__ __noinline__ void bin_add_edge(int b, float w, float vre, float vim, int blo, int b0,
                                          float2* win, int tid, C32* Trow, int nr, int Wt,
                                          unsigned int* err) {
    if (b < 0) {
        if (b != -1) return;
        b = 0;              // x in (-1, 0): truncation gives bin 0 and w = x
        w -= 1.f;
    }
    if (b >= nr) return;
    const float w0 = 1.f - w;
    const bool two = (b + 1) < nr;
    const int sl = b - blo;
    if ((unsigned)sl < (unsigned)(RP_WIN - 1)) {
        float2* p0 = &win[sl * RP_PAIR_THREADS + tid];
        float2 v0 = *p0;
        v0.x = fmaf(vre, w0, v0.x);
        v0.y = fmaf(vim, w0, v0.y);
        *p0 = v0;
        if (two) {
            float2* p1 = p0 + RP_PAIR_THREADS;
            float2 v1 = *p1;
            v1.x = fmaf(vre, w, v1.x);
            v1.y = fmaf(vim, w, v1.y);
            *p1 = v1;
        }
        return;
    }
    const int o0 = b - b0;
    if (o0 >= 0 && o0 < Wt) {
        C32 t0 = Trow[o0];
        t0.x = fmaf(vre, w0, t0.x);
        t0.y = fmaf(vim, w0, t0.y);
        Trow[o0] = t0;
    } else {
        atomicOr(err, 1u);
    }
    if (two) {
        if (o0 + 1 >= 0 && o0 + 1 < Wt) {
            C32 t1 = Trow[o0 + 1];
            t1.x = fmaf(vre, w, t1.x);
            t1.y = fmaf(vim, w, t1.y);
            Trow[o0 + 1] = t1;
        } else {
            atomicOr(err, 1u);
        }
    }
}

// Common case inline (both bins inside the window and the trace); the rest
// (window spill, x < 0, the last bin) in bin_add_edge.
// floor(x) as an integer (cvt.rmi: the conversion unit, not the FP32 pipe).
__device__ __forceinline__ int floor_i(float x) {
    int r;
    asm("cvt.rmi.s32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void bin_add(float xr, float vre, float vim, int blo, int b0,
                                        float2* win, int tid, C32* Trow, const PairArgs& A) {
    const int sl = floor_i(xr);
    const float w = xr - (float)sl;
    const int b = blo + sl;
    if ((unsigned)sl < (unsigned)(RP_WIN - 1) && (unsigned)b < (unsigned)A.nr1) {
        float2* p0 = &win[sl * RP_PAIR_THREADS + tid];
        float2* p1 = p0 + RP_PAIR_THREADS;
        float2 v0 = *p0, v1 = *p1;
        const float w0 = 1.f - w;
        v0.x = fmaf(vre, w0, v0.x);
        v0.y = fmaf(vim, w0, v0.y);
        v1.x = fmaf(vre, w, v1.x);
        v1.y = fmaf(vim, w, v1.y);
        *p0 = v0;
        *p1 = v1;
    } else {
        bin_add_edge(b, w, vre, vim, blo, b0, win, tid, Trow, A.nr, A.Wt, A.err);
    }
}

// bin_add for a chunk whose pairs all fall inside the window and the trace
// (pair_item checks that per chunk and warp): no range tests, no edge path.
// The clamp only keeps a (never expected) stray bin inside the window.
__device__ __forceinline__ void bin_add_fast(float xr, float vre, float vim, float2* win, int tid) {
    const int f = floor_i(xr);
    const float w = xr - (float)f;
    const unsigned sl = min((unsigned)f, (unsigned)(RP_WIN - 2));
    float2* p0 = &win[sl * RP_PAIR_THREADS + tid];
    float2* p1 = p0 + RP_PAIR_THREADS;
    float2 v0 = *p0, v1 = *p1;
    const float w0 = 1.f - w;
    v0.x = fmaf(vre, w0, v0.x);
    v0.y = fmaf(vim, w0, v0.y);
    v1.x = fmaf(vre, w, v1.x);
    v1.y = fmaf(vim, w, v1.y);
    *p0 = v0;
    *p1 = v1;
}

// Dynamic shared memory of the pair kernels: two record buffers, the
// per-thread bin windows, the threads' FP64 target positions.
extern __shared__ __align__(128) unsigned char pair_smem[];
#define RP_PAIR_WIN_OFF (2 * RP_CHUNK * sizeof(FacetRec))
#define RP_PAIR_TPOS_OFF (RP_PAIR_WIN_OFF + (size_t)RP_WIN * RP_PAIR_THREADS * sizeof(float2))
#define RP_PAIR_SMEM_BYTES (RP_PAIR_TPOS_OFF + 3 * RP_PAIR_THREADS * sizeof(double))

template <int NT, int ILP, class PA>
__device__ __forceinline__ void pair_item(const PA& A, int s, int tb, int part, uint64_t* bars, uint32_t* phase) {
    // every hot shared array is derived here from the shared symbol itself
    FacetRec* srec = reinterpret_cast<FacetRec*>(pair_smem);                       // [2][RP_CHUNK]
    float2* win = reinterpret_cast<float2*>(pair_smem + RP_PAIR_WIN_OFF);          // [RP_WIN][threads]
    double* s_tpos = reinterpret_cast<double*>(pair_smem + RP_PAIR_TPOS_OFF);      // [3][threads]
    const int tid = threadIdx.x;
    const int nq = A.ntl[s];
    const int n = A.nill[s];
    if (tb * RP_PAIR_THREADS >= nq || n == 0) return;
    const int nchunks = (n + RP_CHUNK - 1) / RP_CHUNK;
    const int k0 = (int)((int64_t)nchunks * part / RP_PARTS);
    const int k1 = (int)((int64_t)nchunks * (part + 1) / RP_PARTS);
    if (k0 >= k1) return;
    const int q = tb * RP_PAIR_THREADS + tid;
    const bool active = q < nq;
    float tnx = 0, tny = 0, tnz = 1;
    int b0 = 0;
    C32* Trow = nullptr;
    if (active) {
        const int64_t ti = A.tlist[(size_t)s * A.tstride + q];
        s_tpos[tid] = A.TG[ti];
        s_tpos[RP_PAIR_THREADS + tid] = A.TG[A.nt + ti];
        s_tpos[2 * RP_PAIR_THREADS + tid] = A.TG[2 * A.nt + ti];
        tnx = (float)A.TG[3 * A.nt + ti]; tny = (float)A.TG[4 * A.nt + ti];
        tnz = (float)A.TG[5 * A.nt + ti];
        b0 = A.bt0[(size_t)s * A.tstride + q];
        Trow = A.T + (((size_t)part * A.nb + s) * A.tstride + q) * A.Wt;
    }
    const FacetRec* rbase = A.rec + (size_t)s * A.rstride;
    // prologue: stage chunk k0
    if (tid == 0) {
        int cnt = min(RP_CHUNK, n - k0 * RP_CHUNK);
        uint32_t bytes = (uint32_t)(cnt * sizeof(FacetRec));
        mbar_expect_tx(&bars[0], bytes);
        tma_bulk_g2s(srec, rbase + (size_t)k0 * RP_CHUNK, bytes, &bars[0]);
    }
    for (int k = k0; k < k1; ++k) {
        const int buf = (k - k0) & 1;
        // prefetch the next chunk into the other buffer (its readers
        // finished at the trailing __syncthreads of the previous step)
        if (tid == 0 && k + 1 < k1) {
            int cnt = min(RP_CHUNK, n - (k + 1) * RP_CHUNK);
            uint32_t bytes = (uint32_t)(cnt * sizeof(FacetRec));
            mbar_expect_tx(&bars[buf ^ 1], bytes);
            tma_bulk_g2s(srec + (buf ^ 1) * RP_CHUNK, rbase + (size_t)(k + 1) * RP_CHUNK, bytes,
                         &bars[buf ^ 1]);
        }
        const ChunkMeta* mp = A.meta + (size_t)s * A.mstride + k;
        if (!mbar_wait(&bars[buf], phase[buf])) {
            if (tid == 0) atomicOr(A.err + 1, 1u);
        }
        phase[buf] ^= 1u;
        const FacetRec* R = srec + buf * RP_CHUNK;
        Anchor an;
        int blo = 0;
        bool fits = true;
        if (active) {
            // FP64 anchors of this (chunk, target)
            const double mcx = mp->cx, mcy = mp->cy, mcz = mp->cz;
            const double Dx = s_tpos[tid] - mcx, Dy = s_tpos[RP_PAIR_THREADS + tid] - mcy,
                         Dz = s_tpos[2 * RP_PAIR_THREADS + tid] - mcz;
            const double T0 = sqrt(Dx * Dx + Dy * Dy + Dz * Dz);
            const double xt = A.nidx * T0 * A.inv_dr;
            const double tt = A.nidx * T0 * A.inv_lam;
            const double lo = (double)mp->xmin + A.nidx * (T0 - (double)mp->R) * A.inv_dr;
            const double hi = (double)mp->xmax + A.nidx * (T0 + (double)mp->R) * A.inv_dr;
            blo = (int)floor(lo) - 1;
            // every pair's bin x lies in [lo, hi] (triangle inequality on the
            // chunk's bounding radius); with half a bin of margin for FP32
            // rounding, both split bins stay inside the window and the trace
            fits = blo >= 0 && blo + RP_WIN <= A.nr1 && hi + 0.5 < (double)(blo + RP_WIN - 1) &&
                   (double)A.kt * (double)mp->R < 40.0;     // |kt dT| <= kt R: the phase bound
            an.Dx = (float)Dx; an.Dy = (float)Dy; an.Dz = (float)Dz;
            an.T0 = (float)T0; an.T0sq = (float)(T0 * T0);
            an.tau0 = (float)(tt - floor(tt));
            an.xbase = (float)(xt - (double)blo);
            an.tnx = tnx; an.tny = tny; an.tnz = tnz;
            an.eaT0 = (float)((double)A.ealpha * T0);
        }
        const bool all_fit = __all_sync(0xffffffffu, fits);
        if (active) {
            for (int w = 0; w < RP_WIN; ++w) win[w * RP_PAIR_THREADS + tid] = make_float2(0.f, 0.f);
            const int cnt = mp->n;
            const bool prisms = (A.np > 0) && !A.lossless;
            int jj = 0;
            if (all_fit && !prisms) {
                if (ILP == 2)
                for (; jj + 1 < cnt; jj += 2) {
                    const FacetRec r0 = R[jj];
                    const FacetRec r1 = R[jj + 1];
                    float x0, re0, im0, x1, re1, im1;
                    pair_eval<NT, false>(r0, an, A, x0, re0, im0);
                    pair_eval<NT, false>(r1, an, A, x1, re1, im1);
                    bin_add_fast(x0, re0, im0, win, tid);
                    bin_add_fast(x1, re1, im1, win, tid);
                }
                for (; jj < cnt; ++jj) {
                    const FacetRec r0 = R[jj];
                    float x0, re0, im0;
                    pair_eval<NT, false>(r0, an, A, x0, re0, im0);
                    bin_add_fast(x0, re0, im0, win, tid);
                }
            } else {
                if (ILP == 2)
                for (; jj + 1 < cnt; jj += 2) {
                    const FacetRec r0 = R[jj];
                    const FacetRec r1 = R[jj + 1];
                    float x0, re0, im0, x1, re1, im1;
                    pair_eval<NT>(r0, an, A, x0, re0, im0);
                    pair_eval<NT>(r1, an, A, x1, re1, im1);
                    if (prisms) {
                        const float f0 = prism_factor(r0.a, mp->cx, mp->cy, mp->cz, an.Dx, an.Dy, an.Dz, an.T0sq,
                                                      A.PR, A.np, A.ealpha);
                        const float f1 = prism_factor(r1.a, mp->cx, mp->cy, mp->cz, an.Dx, an.Dy, an.Dz, an.T0sq,
                                                      A.PR, A.np, A.ealpha);
                        re0 *= f0; im0 *= f0; re1 *= f1; im1 *= f1;
                    }
                    bin_add(x0, re0, im0, blo, b0, win, tid, Trow, A);
                    bin_add(x1, re1, im1, blo, b0, win, tid, Trow, A);
                }
                for (; jj < cnt; ++jj) {
                    const FacetRec r0 = R[jj];
                    float x0, re0, im0;
                    pair_eval<NT>(r0, an, A, x0, re0, im0);
                    if (prisms) {
                        const float f0 = prism_factor(r0.a, mp->cx, mp->cy, mp->cz, an.Dx, an.Dy, an.Dz, an.T0sq,
                                                      A.PR, A.np, A.ealpha);
                        re0 *= f0; im0 *= f0;
                    }
                    bin_add(x0, re0, im0, blo, b0, win, tid, Trow, A);
                }
            }
            // flush the window into the owned trace
            for (int w = 0; w < RP_WIN; ++w) {
                const float2 v = win[w * RP_PAIR_THREADS + tid];
                if (v.x != 0.f || v.y != 0.f) {
                    const int o = blo + w - b0;
                    if (o >= 0 && o < A.Wt) {
                        C32 t0 = Trow[o];
                        t0.x += v.x;
                        t0.y += v.y;
                        Trow[o] = t0;
                    } else {
                        atomicOr(A.err, 1u);
                    }
                }
            }
        }
        __syncthreads();   // everyone done with buffer `buf` before it is refilled
    }
}

#define RP_PAIR_SMEM_DECL                                                                       \
    __shared__ uint64_t bars[2];                                                                \
    __shared__ unsigned int s_item;                                                             \
    const int tid = threadIdx.x;                                                                \
    if (tid == 0) {                                                                             \
        mbar_init(&bars[0], 1);                                                                 \
        mbar_init(&bars[1], 1);                                                                 \
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");                     \
    }                                                                                           \
    __syncthreads();                                                                            \
    uint32_t phase[2] = {0u, 0u};

#define RP_PAIR_SMEM_END                                                    \
    if (tid == 0) {                                                         \
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&bars[0]))); \
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&bars[1]))); \
    }


// Launch of the multi-job kernel k_pairs32m (rp_multi.cu) in configuration
// cfg over items work items of njobs jobs.
int launch_pairs_multi(int cfg, const PairJob* d_jobs, const unsigned int* d_start, int njobs,
                       unsigned int* d_work, int64_t items, int sms, cudaStream_t st);

}  // namespace rpk
