// rp_pair.cuh -- the pair stage of the fast form, shared by the single-batch
// kernel (rp_fast.cu) and the multi-job kernel (rp_multi.cu): the facet-pair
// record, the TMA bulk staging helpers, the FP32 split-precision evaluation of
// two (facet, target) pairs at once in packed two-lane FP32 instructions
// (compTargetRays, compRefrEnergyIn, accumulateTarget: geometry_kernels.cu:
// 272-350, 520-554, radar_kernels.cu:767-830), the deterministic window
// binning and the body of one work item.
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
#define RP_WIN 16             // bins in a thread's per-chunk window (specular kernel: two windows)
#define RP_WIN_WIDE 24        // the default-mode and ttype-0 kernels' window: a 256-facet chunk of
                              // 2.5 m facets at 12.5 m bins spans up to ~14 bins for one target
#define RP_PARTS 4            // facet-range splits per (trace, target block)
#define RP_LPARTS 2           // log2 RP_PARTS

namespace rpk {

using C32 = Cx<float>;

// Records of two consecutive facets of a chunk, interleaved field by field:
// v[i] = {field 2i of facet 0, field 2i of facet 1, field 2i+1 of facet 0,
// field 2i+1 of facet 1}.  One 128-bit shared-memory load then leaves a
// field of both facets in adjacent registers, the operand of one packed
// two-lane FP32 instruction.  A chunk with an odd count ends with a pair
// whose second facet repeats the first with K = 0 (it adds exact zeros).
// In a scene whose facet frames (n, u, v) are all orthonormal the normal is
// not needed (sin^2 of the incidence angle comes from the tangent
// components) and fields 4 and 5 hold a.u and a.v instead (a = facet -
// chunk centre), field 6 is unused.
enum FacetField {
    F_DX, F_DY, F_DZ, F_Q,      // facet - chunk centre, |facet - chunk centre|^2
    F_NX, F_NY, F_NZ, F_XI,     // normal, xI = (Itd - rst) / dr
    F_UX, F_UY, F_UZ, F_PH,     // u tangent / 2, -2 pi frac(Itd / lam) (radians)
    F_VX, F_VY, F_VZ, F_K,      // v tangent / 2, K = hoisted amplitude factor
    RP_NFIELD,
    F_AU = F_NX, F_AV = F_NY    // orthonormal-frame records
};
struct __align__(16) FacetPair {
    float4 v[RP_NFIELD / 2];
};
#define RP_CHUNK_PAIRS (RP_CHUNK / 2)

// Specular mode: the incident leg's refraction angle Rth and azimuth Iph of
// both facets of a pair, as sines and cosines (facet 0 first in each pair of
// components).  compRefrEnergyIn/Out take facetReradiation of Rth - Tth and
// Iph - Tph (geometry_kernels.cu:527-537, 563-570).
struct __align__(16) FacetSpec {
    float4 r;   // {sin Rth, sin Rth, cos Rth, cos Rth}
    float4 p;   // {cos Iph, cos Iph, sin Iph, sin Iph}
};

// ttype-0 targets (genRefrPhasor): per facet of a pair the trace's constant
// frc^2 nill P Grefr^2 fs^4 / (4 pi)^2 (times (fs^2/lam)^4 in specular mode)
// and Itd in FP32.
struct __align__(16) FacetT0 {
    float4 v;   // {a0, a0, Itd, Itd}
};

// Field f of both facets of a pair.
template <int F>
__device__ __forceinline__ float2 fld(const FacetPair& p) {
    const float4& q = p.v[F >> 1];
    return (F & 1) ? make_float2(q.z, q.w) : make_float2(q.x, q.y);
}

// Packed two-lane FP32 arithmetic (sm_100 and later: one instruction for
// both lanes, each lane rounded exactly as fmaf / __fmul_rn / __fadd_rn).
using f2 = float2;
__device__ __forceinline__ f2 bc(float a) { return make_float2(a, a); }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ f2 mul2(f2 a, f2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ f2 add2(f2 a, f2 b) { return __fadd2_rn(a, b); }
// Negation, folded by the compiler into the consuming packed instruction.
__device__ __forceinline__ f2 neg2(f2 a) { return make_float2(-a.x, -a.y); }

// Per chunk: its centre is the trace origin plus cf, exactly (cf is rounded
// to FP32 first and the centre defined from it), so the pair kernel forms
// the anchor distances in double-float FP32 arithmetic without error from cf.
struct __align__(16) ChunkMeta {
    float cfx, cfy, cfz;   // chunk centre - trace origin (exact)
    float cch, ccl;        // |cf|^2 as a double-float (high, low)
    float lo_off, hi_off;  // xmin - kb R, xmax + kb R: bin bounds relative to n T0 / dr
    int n;                 // facets in the chunk
    float R;               // max |facet - centre|
    float xmin, xmax;      // range of (Itd - rst)/dr
    int phase_ok;          // kt R < 40: the pairs' phase stays within +-42 turns
    double cx, cy, cz;     // chunk centre (FP64: origin + cf)
    double bbmin[3], bbmax[3];
};
static_assert(sizeof(ChunkMeta) % 16 == 0, "ChunkMeta is staged by bulk copies");

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

// Bounded wait on an mbarrier phase: at most `limit` polls; returns false if
// the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase, int limit) {
    for (int it = 0; it < limit; ++it) {
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
    const FacetPair* rec;   // [nb][rstride / 2] facet pairs
    const ChunkMeta* meta;
    const double* org;      // [nb][4] trace origins (FP64)
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
    C32* T;             // [2^lparts][nb][tstride][Wt] row elements, each {high, low} (two C32)
    int Wt;
    int nb;
    int tblocks;        // target blocks per trace
    unsigned int* work; // work counter
    unsigned int* err;  // error flags: [0] window overflow, [1] wait timeout
    int spin_limit;     // polls of a chunk's mbarrier before the wait gives up
    int stall_copies;   // test mode: no bulk copy is issued, so every wait runs out
    // constants
    float nr_f;
    int nr;
    int nr1;            // nr - 1: both split bins are inside the trace when b < nr - 1
    float kb;           // n / dr
    float kt;           // n / lam (turns per metre)
    float kr;           // -2 pi n / lam (radians per metre)
    float pik;          // pi * (pi_F * fs / lam): sinc arguments in radians
    float pik2;         // pik^2
    float sc[8];        // sinc polynomial in t' = a^2 / pik^2 (sinc_poly, scaled)
    float ealpha;       // -2 alpha2 log2(e)
    float eks;          // -2 ks^2 log2(e)
    float kth, ktl;     // n / lam (turns per metre) as a double-float
    float kbh, kbl;     // n / dr (bins per metre) as a double-float
    int lossless;
    // specular mode (k_pairs32s): the inbound and outbound legs differ by
    // their facetReradiation factors and are binned into separate traces
    const FacetSpec* spec;  // [nb][rstride / 2], like rec
    C32* T2;                // outbound-leg parts, laid out like T
    float sr[8];            // sinc polynomial in a^2 / pikr^2, pikr = pi fs / lam (scaled)
    float pikr2;            // pikr^2 (special-function path)
    float e21;              // eps2 / eps1: sin^2 of the outbound Snell angle over sin^2(Tth)
    float s2tir;            // sin^2(1e4): the reference's total-internal-reflection angle
    // ttype-0 targets (pair_item_t0): targets [tq0[s], ntl[s]) of the list
    const FacetT0* t0rec;   // [nb][rstride / 2]
    const int* tq0;
    float kb0;              // c1/c2 / dr: bins per metre of Ttd
    float kb0h, kb0l;       // the same as a double-float
    float kt0h, kt0l;       // 2 turn c1/c2: phase turns per metre of Ttd, double-float
    float kr0;              // 2 pi kt0 (radians per metre)
    int rf;                 // rerad_funct: 0 none, 1-3 angle threshold, 4 Gaussian
    float rcos;             // threshold on cos(TargetTh) for rf 1-3
    float rgl;              // rf 4: -0.5 log2(e) / (pi_F/180)^2
    // log2 of the facet-range parts per (trace, target block): log2 RP_PARTS,
    // more in a wave whose parts are split further (k_pairs32's SUB instance)
    int lparts;
};

// A job of the multi-job pair kernel: a batch's arguments and its sinc
// polynomial degree (0: special-function unit).
struct PairJob {
    PairArgs a;
    int deg;
    int ortho;      // the batch's scene has orthonormal facet frames
};

// Jobs of one k_pairs32mk launch, passed in the parameter space (< 32 KB);
// wi[j]: job j's work-counter index.
#define RP_MAXJ 80
struct PairJobTable {
    PairJob job[RP_MAXJ];
    int wi[RP_MAXJ];
    int njobs;
};
static_assert(sizeof(PairJobTable) <= 32000, "kernel parameters are limited to 32 KB");

// Per-(chunk, target) anchors of the split-precision evaluation.
struct Anchor {
    float Dx, Dy, Dz;     // target - chunk centre (FP32 of an FP64 difference)
    float T0, T0sq;       // |target - chunk centre| (FP64 -> FP32)
    float ph0;            // -2 pi frac(n T0 / lam): phase of the anchor (radians)
    float xbase;          // n T0 / dr - blo (bins, relative to the window start)
    float tnx, tny, tnz;  // target normal
    float nDtn;           // -(target - chunk centre).(target normal)
    float eaT0;           // ealpha T0 (+ eks with orthonormal frames): attenuation exponent at the anchor
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

// sin(a)/a as a degree-D polynomial in t' = a^2 / pik^2 (coefficients
// fitted per scene on a in [0, amax] and scaled, see sinc_poly), Horner
// form, both lanes at once.
template <int D>
__device__ __forceinline__ f2 sinc_poly2(const float* c, f2 t) {
    f2 s = fma2(bc(c[D]), t, bc(c[D - 1]));
#pragma unroll
    for (int k = D - 2; k >= 0; --k) s = fma2(s, t, bc(c[k]));
    return s;
}

// sin(a)/a for a^2 = u through the special-function unit; 1 for |a| < pi
// 1e-6 (elementary_kernels.cu:50-53).  Returns the sine and the divisor
// separately so four factors share one division.
__device__ __forceinline__ void sinc_sfu(float u, float& num, float& den) {
    const float a = u > 0.f ? u * rsqrt_a(u) : 0.f;
    const bool z = a < 3.14159265e-6f;
    num *= z ? 1.f : __sinf(a);
    den *= z ? 1.f : a;
}

// Two (facet, target) evaluations of the target leg (compTargetRays,
// compRefrEnergyIn, accumulateTarget; geometry_kernels.cu:272-350, 520-554,
// radar_kernels.cu:767-830): the two facets of pair record r against one
// target, in packed two-lane FP32.  Returns per lane the phasor's amplitude,
// the cosine and sine of its phase, and x - blo, the bin coordinate relative
// to the window start (pair_eval2 below forms the phasor itself).
//
// The two directivities facet_G(Tth, Tph) and facet_G(TargetTh, Tph)
// (radar_kernels.cu:658-677) need sinc(pik/pi * sin(th) cos(ph)) and
// sinc(pik/pi * sin(th) sin(ph)), sinc(x) = sin(pi x)/(pi x).  The direction
// e = facet - target is not normalised: with its dot products pb = e.n,
// pt = e.n_target, pc = e.u, pd = e.v and d2 = |e|^2, sin^2(th) = 1 -
// pb^2/d2 (likewise with pt) and cos^2(ph) = xs = pd^2 / (pc^2 + pd^2),
// sin^2(ph) = 1 - xs, so the four squared arguments over pik^2 are
// sin^2(th) xs and sin^2(th) (1 - xs) per angle.  A tiny constant in both
// sums of xs gives xs = 1 when pc = pd = 0 (atan2(0, 0) = 0: cos = 1), and
// changes nothing measurable otherwise.  1 - c^2 may round a hair below 0
// for |c| ~ 1: harmless in the polynomial, clamped for the SFU path.  NT > 0
// evaluates sin(a)/a as a polynomial in a^2; NT == 0 uses the SFU.
// RED: reduce the phase to [-pi, pi] before the special-function sine and
// cosine; the fast path skips it when the chunk keeps |phase| below 84 pi
// (sin/cos.approx hold their accuracy over +-100 pi radians).
template <int NT, bool ORTHO, bool RED = true>
__device__ __forceinline__ void pair_eval2_core(const FacetPair& r, const Anchor& an, const PairArgs& A, f2& xr,
                                                f2& amp_out, f2& cs, f2& sn) {
    const f2 ONE = bc(1.f), M1 = bc(-1.f);
    const f2 dx = fld<F_DX>(r), dy = fld<F_DY>(r), dz = fld<F_DZ>(r);
    // m = -2 D: Ttd^2 - T0^2 = |a|^2 - 2 D.a as one chain from |a|^2; the
    // record's tangents are halved (exactly), so m.(u/2) = -D.u
    const f2 mx = bc(-2.f * an.Dx), my = bc(-2.f * an.Dy), mz = bc(-2.f * an.Dz);
    const f2 qd = fma2(mx, dx, fma2(my, dy, fma2(mz, dz, fld<F_Q>(r))));   // Ttd^2 - T0^2
    const f2 d2 = add2(bc(an.T0sq), qd);
    const f2 rinv = make_float2(rsqrt_a(d2.x), rsqrt_a(d2.y));
    const f2 sT = fma2(d2, rinv, bc(an.T0));                     // Ttd + T0
    const f2 dT = mul2(qd, make_float2(rcp_a(sT.x), rcp_a(sT.y)));   // Ttd - T0 without cancellation
    // t1..t4: the four squared sinc arguments over pik^2; aT = sin^2(Tth)
    f2 aT, t1, t2, t3, t4;
    if (ORTHO) {
        // e = a - D: e.u = a.u - D.u etc. (a.u, a.v from the record), and
        // sin^2(Tth) cos^2(Tph) = (e.v)^2 / d2, sin^2(Tth) sin^2(Tph) =
        // (e.u)^2 / d2 because n, u, v are orthonormal
        const f2 pc = fma2(mx, fld<F_UX>(r), fma2(my, fld<F_UY>(r), fma2(mz, fld<F_UZ>(r), fld<F_AU>(r))));
        const f2 pd = fma2(mx, fld<F_VX>(r), fma2(my, fld<F_VY>(r), fma2(mz, fld<F_VZ>(r), fld<F_AV>(r))));
        const f2 pt = fma2(dx, bc(an.tnx), fma2(dy, bc(an.tny), fma2(dz, bc(an.tnz), bc(an.nDtn))));
        const f2 pcr = mul2(pc, rinv), pdr = mul2(pd, rinv), ptr = mul2(pt, rinv);
        t1 = fma2(pdr, pdr, bc(1e-30f));
        t2 = mul2(pcr, pcr);
        aT = add2(t1, t2);
        const f2 xs = mul2(t1, make_float2(rcp_a(aT.x), rcp_a(aT.y)));
        const f2 aD = fma2(ptr, neg2(ptr), ONE);
        t3 = mul2(aD, xs);
        t4 = fma2(t3, M1, aD);
    } else {
        // e = facet - target; only squares of its dot products enter (and
        // the in-plane split is a ratio, so the halved tangents cancel)
        const f2 hf = bc(0.5f);
        const f2 ex = fma2(mx, hf, dx), ey = fma2(my, hf, dy), ez = fma2(mz, hf, dz);
        const f2 pb = fma2(ex, fld<F_NX>(r), fma2(ey, fld<F_NY>(r), mul2(ez, fld<F_NZ>(r))));
        const f2 pt = fma2(ex, bc(an.tnx), fma2(ey, bc(an.tny), mul2(ez, bc(an.tnz))));
        const f2 pc = fma2(ex, fld<F_UX>(r), fma2(ey, fld<F_UY>(r), mul2(ez, fld<F_UZ>(r))));
        const f2 pd = fma2(ex, fld<F_VX>(r), fma2(ey, fld<F_VY>(r), mul2(ez, fld<F_VZ>(r))));
        const f2 pbr = mul2(pb, rinv), ptr = mul2(pt, rinv);
        aT = fma2(pbr, neg2(pbr), ONE);
        const f2 aD = fma2(ptr, neg2(ptr), ONE);
        const f2 X = fma2(pd, pd, bc(1e-30f));
        const f2 h2 = fma2(pc, pc, X);
        const f2 xs = mul2(X, make_float2(rcp_a(h2.x), rcp_a(h2.y)));
        t1 = mul2(aT, xs); t3 = mul2(aD, xs);
        t2 = fma2(t1, M1, aT); t4 = fma2(t3, M1, aD);
    }
    f2 S;
    if (NT > 0) {
        constexpr int D = NT > 0 ? NT : 1;
        S = mul2(mul2(sinc_poly2<D>(A.sc, t1), sinc_poly2<D>(A.sc, t2)),
                 mul2(sinc_poly2<D>(A.sc, t3), sinc_poly2<D>(A.sc, t4)));
        if (NT >= 5) S = make_float2(fabsf(S.x), fabsf(S.y));   // sinc changes sign beyond a = pi
    } else {
        const f2 P2 = bc(A.pik2);
        const f2 u1 = mul2(t1, P2), u2 = mul2(t2, P2), u3 = mul2(t3, P2), u4 = mul2(t4, P2);
        float n0 = 1.f, e0 = 1.f, n1 = 1.f, e1 = 1.f;
        sinc_sfu(u1.x, n0, e0); sinc_sfu(u2.x, n0, e0); sinc_sfu(u3.x, n0, e0); sinc_sfu(u4.x, n0, e0);
        sinc_sfu(u1.y, n1, e1); sinc_sfu(u2.y, n1, e1); sinc_sfu(u3.y, n1, e1); sinc_sfu(u4.y, n1, e1);
        S = make_float2(fabsf(__fdividef(n0, e0)), fabsf(__fdividef(n1, e1)));
    }
    // attenuation and roughness (zero constants when lossless); ealpha Ttd
    // = ealpha T0 + ealpha (Ttd - T0), eks cos^2(Tth) = eks - eks sin^2(Tth)
    // (the eks term is part of the anchor's eaT0)
    const f2 e2 = fma2(bc(-A.eks), aT, fma2(bc(A.ealpha), dT, bc(an.eaT0)));
    const f2 amp = mul2(mul2(fld<F_K>(r), S), mul2(rinv, make_float2(ex2_a(e2.x), ex2_a(e2.y))));
    f2 ph = fma2(bc(A.kr), dT, add2(fld<F_PH>(r), bc(an.ph0)));
    if (RED) {
        const f2 k = mul2(ph, bc(0.159154943091895336f));
        ph = fma2(make_float2(rintf(k.x), rintf(k.y)), bc(-6.28318530717958647f), ph);
    }
    __sincosf(ph.x, &sn.x, &cs.x);
    __sincosf(ph.y, &sn.y, &cs.y);
    amp_out = amp;
    xr = fma2(bc(A.kb), dT, add2(fld<F_XI>(r), bc(an.xbase)));
}

// pair_eval2_core with the phasor formed: vre + i vim = amp e^{i ph}.
template <int NT, bool ORTHO, bool RED = true>
__device__ __forceinline__ void pair_eval2(const FacetPair& r, const Anchor& an, const PairArgs& A, f2& xr,
                                           f2& vre, f2& vim) {
    f2 amp, cs, sn;
    pair_eval2_core<NT, ORTHO, RED>(r, an, A, xr, amp, cs, sn);
    vre = mul2(amp, cs);
    vim = mul2(amp, sn);
}

// pair_eval2 for specular mode (general frames): also returns per lane the
// facetReradiation amplitudes of the two refraction legs, g1 (inbound:
// Rth - Tth, Iph - Tph) and g2 (outbound: the Snell angle of pi_F - Tth from
// eps2 to eps1, Tph - Iph), each |sinc * sinc| with sinc(x) = sin(pi x)/(pi x)
// of (fs/lam) sin(th) cos(ph) and (fs/lam) sin(th) sin(ph); the constant
// fs^2/lam is part of the record's K.  From the dot products of e = facet -
// target: cos Tth = e.n / |e|, sin Tth = sqrt(1 - cos^2), and (cos Tph, sin
// Tph) = -(e.v, e.u) / |(e.v, e.u)|, so cos(Iph - Tph) and sin(Iph - Tph)
// follow from the record's sines and cosines without angles.  A shift of e.v
// by -1e-15 (below FP32 resolution for any other value) gives cos Tph = 1 at
// e.u = e.v = 0, as atan2(0, 0) = 0 does.  Beyond total internal reflection
// the reference's flag angle 1e4 gives sin^2(1e4).
// The two reradiation amplitudes g1, g2 of pair_eval2s from cos Tth = pbr,
// sin^2 Tth = aT, the in-plane components pc, pd (pd already shifted) and
// rh = 1 / (pc^2 + pd^2).
template <int NT>
__device__ __forceinline__ void spec_rerad2(const FacetSpec& sp, const PairArgs& A, f2 pbr, f2 aT, f2 pc, f2 pd,
                                            f2 rh, f2& g1, f2& g2) {
    const f2 sR = make_float2(sp.r.x, sp.r.y), cR = make_float2(sp.r.z, sp.r.w);
    const f2 cI = make_float2(sp.p.x, sp.p.y), sI = make_float2(sp.p.z, sp.p.w);
    const f2 aTc = make_float2(fmaxf(aT.x, 1e-30f), fmaxf(aT.y, 1e-30f));
    const f2 sTh = mul2(aTc, make_float2(rsqrt_a(aTc.x), rsqrt_a(aTc.y)));
    const f2 st1 = fma2(sR, pbr, mul2(neg2(cR), sTh));
    const f2 q1 = mul2(st1, st1);
    const f2 q2r = mul2(bc(A.e21), aT);
    const f2 q2 = make_float2(q2r.x > 1.f ? A.s2tir : q2r.x, q2r.y > 1.f ? A.s2tir : q2r.y);
    const f2 cn = fma2(cI, pd, mul2(sI, pc));
    const f2 sn = fma2(sI, pd, mul2(neg2(cI), pc));
    const f2 cc = mul2(mul2(cn, cn), rh), ss = mul2(mul2(sn, sn), rh);
    const f2 u1 = mul2(q1, cc), u2 = mul2(q1, ss), u3 = mul2(q2, cc), u4 = mul2(q2, ss);
    if (NT > 0) {
        constexpr int D = NT > 0 ? NT : 1;
        g1 = mul2(sinc_poly2<D>(A.sr, u1), sinc_poly2<D>(A.sr, u2));
        g2 = mul2(sinc_poly2<D>(A.sr, u3), sinc_poly2<D>(A.sr, u4));
        if (NT >= 5) {
            g1 = make_float2(fabsf(g1.x), fabsf(g1.y));
            g2 = make_float2(fabsf(g2.x), fabsf(g2.y));
        }
    } else {
        const f2 R2 = bc(A.pikr2);
        const f2 v1 = mul2(u1, R2), v2 = mul2(u2, R2), v3 = mul2(u3, R2), v4 = mul2(u4, R2);
        float a0 = 1.f, b0 = 1.f, a1 = 1.f, b1 = 1.f, c0 = 1.f, d0 = 1.f, c1 = 1.f, d1 = 1.f;
        sinc_sfu(v1.x, a0, b0); sinc_sfu(v2.x, a0, b0); sinc_sfu(v1.y, a1, b1); sinc_sfu(v2.y, a1, b1);
        sinc_sfu(v3.x, c0, d0); sinc_sfu(v4.x, c0, d0); sinc_sfu(v3.y, c1, d1); sinc_sfu(v4.y, c1, d1);
        g1 = make_float2(fabsf(__fdividef(a0, b0)), fabsf(__fdividef(a1, b1)));
        g2 = make_float2(fabsf(__fdividef(c0, d0)), fabsf(__fdividef(c1, d1)));
    }
}

template <int NT, bool RED = true>
__device__ __forceinline__ void pair_eval2s(const FacetPair& r, const FacetSpec& sp, const Anchor& an,
                                            const PairArgs& A, f2& xr, f2& vre, f2& vim, f2& g1, f2& g2) {
    const f2 ONE = bc(1.f), M1 = bc(-1.f);
    const f2 dx = fld<F_DX>(r), dy = fld<F_DY>(r), dz = fld<F_DZ>(r);
    const f2 mx = bc(-2.f * an.Dx), my = bc(-2.f * an.Dy), mz = bc(-2.f * an.Dz);
    const f2 qd = fma2(mx, dx, fma2(my, dy, fma2(mz, dz, fld<F_Q>(r))));   // Ttd^2 - T0^2
    const f2 d2 = add2(bc(an.T0sq), qd);
    const f2 rinv = make_float2(rsqrt_a(d2.x), rsqrt_a(d2.y));
    const f2 sT = fma2(d2, rinv, bc(an.T0));
    const f2 dT = mul2(qd, make_float2(rcp_a(sT.x), rcp_a(sT.y)));
    const f2 hf = bc(0.5f);
    const f2 ex = fma2(mx, hf, dx), ey = fma2(my, hf, dy), ez = fma2(mz, hf, dz);
    const f2 pb = fma2(ex, fld<F_NX>(r), fma2(ey, fld<F_NY>(r), mul2(ez, fld<F_NZ>(r))));
    const f2 pt = fma2(ex, bc(an.tnx), fma2(ey, bc(an.tny), mul2(ez, bc(an.tnz))));
    const f2 pc = fma2(ex, fld<F_UX>(r), fma2(ey, fld<F_UY>(r), mul2(ez, fld<F_UZ>(r))));
    const f2 pd = add2(fma2(ex, fld<F_VX>(r), fma2(ey, fld<F_VY>(r), mul2(ez, fld<F_VZ>(r)))), bc(-1e-15f));
    const f2 pbr = mul2(pb, rinv), ptr = mul2(pt, rinv);
    const f2 aT = fma2(pbr, neg2(pbr), ONE);
    const f2 aD = fma2(ptr, neg2(ptr), ONE);
    const f2 X = mul2(pd, pd);
    const f2 h2 = fma2(pc, pc, X);
    const f2 rh = make_float2(rcp_a(h2.x), rcp_a(h2.y));
    const f2 xs = mul2(X, rh);
    const f2 t1 = mul2(aT, xs), t3 = mul2(aD, xs);
    const f2 t2 = fma2(t1, M1, aT), t4 = fma2(t3, M1, aD);
    // the reradiation legs (spec_rerad2)
    spec_rerad2<NT>(sp, A, pbr, aT, pc, pd, rh, g1, g2);
    f2 S;
    if (NT > 0) {
        constexpr int D = NT > 0 ? NT : 1;
        S = mul2(mul2(sinc_poly2<D>(A.sc, t1), sinc_poly2<D>(A.sc, t2)),
                 mul2(sinc_poly2<D>(A.sc, t3), sinc_poly2<D>(A.sc, t4)));
        if (NT >= 5) S = make_float2(fabsf(S.x), fabsf(S.y));
    } else {
        const f2 P2 = bc(A.pik2);
        const f2 w1 = mul2(t1, P2), w2 = mul2(t2, P2), w3 = mul2(t3, P2), w4 = mul2(t4, P2);
        float n0 = 1.f, e0 = 1.f, n1 = 1.f, e1 = 1.f;
        sinc_sfu(w1.x, n0, e0); sinc_sfu(w2.x, n0, e0); sinc_sfu(w3.x, n0, e0); sinc_sfu(w4.x, n0, e0);
        sinc_sfu(w1.y, n1, e1); sinc_sfu(w2.y, n1, e1); sinc_sfu(w3.y, n1, e1); sinc_sfu(w4.y, n1, e1);
        S = make_float2(fabsf(__fdividef(n0, e0)), fabsf(__fdividef(n1, e1)));
    }
    const f2 e2 = fma2(bc(-A.eks), aT, fma2(bc(A.ealpha), dT, bc(an.eaT0)));
    const f2 amp = mul2(mul2(fld<F_K>(r), S), mul2(rinv, make_float2(ex2_a(e2.x), ex2_a(e2.y))));
    f2 ph = fma2(bc(A.kr), dT, add2(fld<F_PH>(r), bc(an.ph0)));
    if (RED) {
        const f2 k = mul2(ph, bc(0.159154943091895336f));
        ph = fma2(make_float2(rintf(k.x), rintf(k.y)), bc(-6.28318530717958647f), ph);
    }
    f2 sn2, cs2;
    __sincosf(ph.x, &sn2.x, &cs2.x);
    __sincosf(ph.y, &sn2.y, &cs2.y);
    vre = mul2(amp, cs2);
    vim = mul2(amp, sn2);
    xr = fma2(bc(A.kb), dT, add2(fld<F_XI>(r), bc(an.xbase)));
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

// Knuth's TwoSum: s = fl(a + b) and its exact rounding error e (a + b = s + e
// exactly); the _rn intrinsics keep the compiler from contracting or
// reordering it.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fadd_rn(s, -a);
    e = __fadd_rn(__fadd_rn(a, -__fadd_rn(s, -bb)), __fadd_rn(b, -bb));
}

// Compensated (Kahan-Babuska) accumulation into a target row element: the
// element is {high, low}, one 16-byte word (two C32 at Trow[2 o],
// Trow[2 o + 1]); each add rounds into the high part and its exact rounding
// error goes into the low part, so high + low carries the sum of every flush
// to about FP32 precision of the sum, however many chunks flush into it.
// Readers take high + low.
__device__ __forceinline__ float4 comp_add(float4 t, float vre, float vim) {
    float s, e;
    two_sum(t.x, vre, s, e);
    t.x = s;
    t.z = __fadd_rn(t.z, e);
    two_sum(t.y, vim, s, e);
    t.y = s;
    t.w = __fadd_rn(t.w, e);
    return t;
}
__device__ __forceinline__ void comp_add_row(C32* Trow, int o, float vre, float vim) {
    float4* p = reinterpret_cast<float4*>(Trow) + o;
    *p = comp_add(*p, vre, vim);
}

// Add one phasor into the thread's window (or, outside it, directly into the
// thread's own trace row, compensated).  Bin and weight follow the reference's two-bin
// split: b = (short)x (truncation), w = x - b (radar_kernels.cu:736-760).
// floor(xr) comes from rounding xr - 1/2 with the 1.5 * 2^23 magic number
// (an exact half rounds either way; the split is continuous there, so both
// give the same contributions); x in (-1, 0) is truncated to bin 0 as the
// reference does.
template <int W>
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
    if ((unsigned)sl < (unsigned)(W - 1)) {
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
        comp_add_row(Trow, o0, vre * w0, vim * w0);
    } else {
        atomicOr(err, 1u);
    }
    if (two) {
        if (o0 + 1 >= 0 && o0 + 1 < Wt) {
            comp_add_row(Trow, o0 + 1, vre * w, vim * w);
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

template <int W>
__device__ __forceinline__ void bin_add(float xr, float vre, float vim, int blo, int b0,
                                        float2* win, int tid, C32* Trow, const PairArgs& A) {
    const int sl = floor_i(xr);
    const float w = xr - (float)sl;
    const int b = blo + sl;
    if ((unsigned)sl < (unsigned)(W - 1) && (unsigned)b < (unsigned)A.nr1) {
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
        bin_add_edge<W>(b, w, vre, vim, blo, b0, win, tid, Trow, A.nr, A.Wt, A.err);
    }
}

// Both lanes' bins, floor(x), without the conversion unit: x + 1.5 2^23
// rounded down lies in [2^23, 2^24), where the FP32 grid is the integers, so
// it is 1.5 2^23 + floor(x) exactly for |x| < 2^22, and its bit pattern is
// 0x4B400000 + floor(x).  fl = floor(x) as floats (exact); s0, s1 = the
// slots, floor(x) clamped to [0, HI] by one unsigned min.  Anything else
// (x < 0, |x| >= 2^22, NaN) lands in slot HI, and no slot leaves the window.
template <unsigned HI>
__device__ __forceinline__ void floor_slots2(f2 x, f2& fl, unsigned& s0, unsigned& s1) {
    const f2 M = bc(12582912.f);
    const f2 t = __fadd2_rd(x, M);
    fl = add2(t, neg2(M));
    s0 = min(__float_as_uint(t.x) - 0x4B400000u, HI);
    s1 = min(__float_as_uint(t.y) - 0x4B400000u, HI);
}

// Adds (v0 += a0 (c, s), v1 += a1 (c, s)) to the window bins of slot sl and
// sl + 1 of the thread whose column starts at wt = win + tid.
__device__ __forceinline__ void win_add2(float2* wt, unsigned sl, float c, float s, float a0, float a1) {
    float2* p0 = wt + sl * RP_PAIR_THREADS;
    float2* p1 = p0 + RP_PAIR_THREADS;
    float2 v0 = *p0, v1 = *p1;
    v0.x = fmaf(c, a0, v0.x);
    v0.y = fmaf(s, a0, v0.y);
    v1.x = fmaf(c, a1, v1.x);
    v1.y = fmaf(s, a1, v1.y);
    *p0 = v0;
    *p1 = v1;
}

// bin_add for the two lanes of a pair evaluation in a chunk whose pairs all
// fall inside the window and the trace (pair_item checks that per chunk and
// warp): no range tests, no edge path, lane 0 before lane 1.  The clamp only
// keeps a (never expected) stray bin inside the window.  The phasor comes as
// its amplitude and direction: the split weights take the amplitude (amp w
// and amp - amp w, one product fewer than forming the phasor first), then
// multiply cos and sin.
template <int W>
__device__ __forceinline__ void bin_add_fast2a(f2 xr, f2 amp, f2 cs, f2 sn, float2* win, int tid) {
    const int f0 = floor_i(xr.x), f1 = floor_i(xr.y);
    const unsigned s0 = min((unsigned)f0, (unsigned)(W - 2)), s1 = min((unsigned)f1, (unsigned)(W - 2));
    const f2 w = fma2(make_float2((float)f0, (float)f1), bc(-1.f), xr);
    const f2 a1 = mul2(amp, w);
    const f2 a0 = add2(amp, neg2(a1));
    float2* const wt = win + tid;
    win_add2(wt, s0, cs.x, sn.x, a0.x, a1.x);
    win_add2(wt, s1, cs.y, sn.y, a0.y, a1.y);
}

// The same bins and split weights in specular mode: the inbound phasor
// times g1 into win and the outbound one times g2 into win2.
__device__ __forceinline__ void bin_add_fast2s(f2 xr, f2 vre, f2 vim, f2 g1, f2 g2, float2* win, float2* win2,
                                               int tid) {
    f2 fl;
    unsigned s0, s1;
    floor_slots2<RP_WIN - 2>(xr, fl, s0, s1);
    const f2 w = fma2(fl, bc(-1.f), xr);
    const f2 w0 = fma2(w, bc(-1.f), bc(1.f));
    const f2 ar = mul2(vre, g1), ai = mul2(vim, g1), br = mul2(vre, g2), bi = mul2(vim, g2);
    float2* const wt = win + tid;
    float2* const wt2 = win2 + tid;
    win_add2(wt, s0, ar.x, ai.x, w0.x, w.x);
    win_add2(wt2, s0, br.x, bi.x, w0.x, w.x);
    win_add2(wt, s1, ar.y, ai.y, w0.y, w.y);
    win_add2(wt2, s1, br.y, bi.y, w0.y, w.y);
}

// One ttype-0 phasor into the thread's window, or (outside it) its target
// row: the whole phasor in the truncated bin (genRefrPhasor +
// genPhasorTrace, radar_kernels.cu:351-398, 401-448); x in (-1, 0) gives bin
// 0, bins outside the trace are dropped.
template <int W>
__device__ __forceinline__ void bin_add1(float xr, float vre, float vim, int blo, int b0, float2* win, int tid,
                                         C32* Trow, const PairArgs& A) {
    const int sl = floor_i(xr);
    int b = blo + sl;
    if ((unsigned)sl < (unsigned)W && (unsigned)b < (unsigned)A.nr) {
        float2* p0 = &win[sl * RP_PAIR_THREADS + tid];
        float2 v0 = *p0;
        v0.x += vre;
        v0.y += vim;
        *p0 = v0;
        return;
    }
    if (b < 0) {
        if (b != -1) return;
        b = 0;
    }
    if (b >= A.nr) return;
    const int sw = b - blo;
    if ((unsigned)sw < (unsigned)W) {
        float2* p0 = &win[sw * RP_PAIR_THREADS + tid];
        float2 v0 = *p0;
        v0.x += vre;
        v0.y += vim;
        *p0 = v0;
        return;
    }
    const int o = b - b0;
    if (o >= 0 && o < A.Wt) {
        comp_add_row(Trow, o, vre, vim);
    } else {
        atomicOr(A.err, 1u);
    }
}

// Flush a thread's bin window into its target's row: each non-zero bin adds
// to the row element it covers, compensated (comp_add: the rounding error of
// the add goes into the element's low part); outside the row: the
// window-overflow flag.  In groups of 8 bins, every row load of a group
// (high and low parts) is issued before its first add, so the
// read-modify-writes overlap instead of waiting on one another.
template <int W>
__device__ __forceinline__ void flush_window(const float2* win, int tid, int blo, int b0, C32* Trow, int Wt,
                                             unsigned int* err) {
    static_assert(W % 8 == 0, "windows flush in groups of 8 bins");
    float4* const R = reinterpret_cast<float4*>(Trow);
#pragma unroll
    for (int g = 0; g < W; g += 8) {
        float2 v[8];
        float4 t[8];
#pragma unroll
        for (int w = 0; w < 8; ++w) v[w] = win[(g + w) * RP_PAIR_THREADS + tid];
#pragma unroll
        for (int w = 0; w < 8; ++w) {
            const int o = blo + g + w - b0;
            const bool nz = v[w].x != 0.f || v[w].y != 0.f;
            t[w] = (nz && o >= 0 && o < Wt) ? R[o] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int w = 0; w < 8; ++w) {
            if (v[w].x != 0.f || v[w].y != 0.f) {
                const int o = blo + g + w - b0;
                if (o >= 0 && o < Wt) {
                    R[o] = comp_add(t[w], v[w].x, v[w].y);
                } else {
                    atomicOr(err, 1u);
                }
            }
        }
    }
}

// ------------------------------------------------ double-float anchors --
// Error-free transformation (FMA TwoProduct; TwoSum is above); the _rn
// intrinsics keep the compiler from contracting it.
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
    p = __fmul_rn(a, b);
    e = __fmaf_rn(a, b, -p);
}

// T0 = |t' - cf| for t' = th + tl (double-float) and an exact FP32 cf, from
// T0^2 = |t'|^2 - 2 t'.cf + |cf|^2 carried as double-floats and one Newton
// correction of the FP32 square root: Th + Tl to ~1e-13 relative; Qh = T0^2
// rounded to FP32.
__device__ __forceinline__ void anchor_distance(float4 th, float4 tl, float cfx, float cfy, float cfz,
                                                float cch, float ccl, float& Th, float& Tl, float& Qh) {
    float px, ex, py, ey, pz, ez;
    two_prod(th.x, cfx, px, ex);
    two_prod(th.y, cfy, py, ey);
    two_prod(th.z, cfz, pz, ez);
    float s1, r1, s2, r2;
    two_sum(px, py, s1, r1);
    two_sum(s1, pz, s2, r2);
    const float dl = __fadd_rn(__fadd_rn(__fadd_rn(ex, ey), __fadd_rn(ez, r1)),
                               __fadd_rn(r2, __fmaf_rn(tl.x, cfx, __fmaf_rn(tl.y, cfy, __fmul_rn(tl.z, cfz)))));
    // Q = |t'|^2 - 2 (s2 + dl) + |cf|^2
    float a1, r3, a2, r4;
    two_sum(th.w, __fmul_rn(-2.f, s2), a1, r3);
    two_sum(a1, cch, a2, r4);
    const float ql = __fadd_rn(__fadd_rn(__fmaf_rn(-2.f, dl, tl.w), ccl), __fadd_rn(r3, r4));
    Qh = __fadd_rn(a2, ql);
    const float Ql = __fadd_rn(ql, -__fadd_rn(Qh, -a2));
    // sqrt: s = Qh rsqrt(Qh), then T0 = s + (Q - s^2) / (2 s)
    const float y = rsqrt_a(Qh);
    const float sq = __fmul_rn(Qh, y);
    float ss, sse;
    two_prod(sq, sq, ss, sse);
    const float res = __fadd_rn(__fadd_rn(__fadd_rn(Qh, -ss), -sse), Ql);
    const float corr = __fmul_rn(res, __fmul_rn(0.5f, y));
    Th = __fadd_rn(sq, corr);
    Tl = __fadd_rn(corr, -__fadd_rn(Th, -sq));
}

// frac((Th + Tl) (kh + kl)) in about [-1/2, 1/2]: the high product exactly
// (its integer part removed exactly), plus the low terms.
__device__ __forceinline__ float frac_dd(float Th, float Tl, float kh, float kl) {
    float p, e;
    two_prod(Th, kh, p, e);
    const float lo = __fadd_rn(e, __fmaf_rn(Th, kl, __fmul_rn(Tl, kh)));
    return __fadd_rn(__fadd_rn(p, -rintf(p)), lo);
}

// (Th + Tl) (kh + kl) = xi + xf with xi = floor of the high product.
__device__ __forceinline__ int floor_dd(float Th, float Tl, float kh, float kl, float& xf) {
    float p, e;
    two_prod(Th, kh, p, e);
    const float lo = __fadd_rn(e, __fmaf_rn(Th, kl, __fmul_rn(Tl, kh)));
    const float fl = floorf(p);
    xf = __fadd_rn(__fadd_rn(p, -fl), lo);
    return (int)fl;
}

// Dynamic shared memory of the pair kernels: two record buffers, the
// per-thread bin windows, the threads' target positions relative to the
// trace origin as double-floats, the two staged chunks' metadata.
extern __shared__ __align__(128) unsigned char pair_smem[];
// Offsets for a window of W bins.
__host__ __device__ constexpr size_t pair_win_off() { return 2 * RP_CHUNK_PAIRS * sizeof(FacetPair); }
__host__ __device__ constexpr size_t pair_tpos_off(int W) { return pair_win_off() + (size_t)W * RP_PAIR_THREADS * sizeof(float2); }
__host__ __device__ constexpr size_t pair_meta_off(int W) { return pair_tpos_off(W) + 2 * RP_PAIR_THREADS * sizeof(float4); }
__host__ __device__ constexpr size_t pair_smem_bytes(int W) { return pair_meta_off(W) + 2 * sizeof(ChunkMeta); }
// specular mode (window RP_WIN) adds the outbound window and two staged
// FacetSpec chunks
#define RP_PAIR_WIN2_OFF pair_smem_bytes(RP_WIN)
#define RP_PAIR_SPEC_OFF (RP_PAIR_WIN2_OFF + (size_t)RP_WIN * RP_PAIR_THREADS * sizeof(float2))
#define RP_PAIR_SPEC_SMEM_BYTES (RP_PAIR_SPEC_OFF + 2 * RP_CHUNK_PAIRS * sizeof(FacetSpec))
static_assert(RP_PAIR_SPEC_OFF % 16 == 0, "FacetSpec chunks are staged by bulk copies");
static_assert(pair_smem_bytes(RP_WIN_WIDE) % 16 == 0, "FacetT0 chunks are staged by bulk copies");

// A wait on a chunk's staged copy that ran out ends the block's work.  The
// thread whose wait ran out skips the chunk (it never reads the unfilled
// buffer); the chunk's trailing barrier tells every thread (a reduction in
// place of the plain barrier, so the common path keeps one barrier per
// chunk); then thread 0 raises the timeout flag (RP_ERR_TIMEOUT on the host)
// and waits, again bounded, for the copies the block still has in flight,
// and the block stops taking work.
__device__ __forceinline__ void abort_block(const PairArgs& A, uint64_t* bars, const uint32_t* phase, int buf,
                                            bool got, bool next_issued) {
    if (threadIdx.x == 0) {
        atomicOr(A.err + 1, 1u);
        if (!A.stall_copies) {
            if (!got) mbar_wait(&bars[buf], phase[buf], A.spin_limit);
            if (next_issued) mbar_wait(&bars[buf ^ 1], phase[buf ^ 1], A.spin_limit);
        }
    }
}

// One work item of the pair kernels; false when a chunk's wait ran out (the
// kernel then stops taking items).
template <int NT, int ILP, bool ORTHO, bool SPEC, int W, class PA>
__device__ __forceinline__ bool pair_item(const PA& A, int s, int tb, int part, uint64_t* bars, uint32_t* phase,
                                          int lparts = RP_LPARTS) {
    static_assert(!SPEC || W == RP_WIN, "the specular layout holds two RP_WIN windows");
    // every hot shared array is derived here from the shared symbol itself
    FacetPair* srec = reinterpret_cast<FacetPair*>(pair_smem);                     // [2][RP_CHUNK_PAIRS]
    float2* win = reinterpret_cast<float2*>(pair_smem + pair_win_off());           // [W][threads]
    float4* s_tq = reinterpret_cast<float4*>(pair_smem + pair_tpos_off(W));        // [2][threads]
    ChunkMeta* smeta = reinterpret_cast<ChunkMeta*>(pair_smem + pair_meta_off(W));  // [2]
    float2* win2 = nullptr;                                                         // [W][threads]
    FacetSpec* sspec = nullptr;                                                     // [2][RP_CHUNK_PAIRS]
    if constexpr (SPEC) {
        win2 = reinterpret_cast<float2*>(pair_smem + RP_PAIR_WIN2_OFF);
        sspec = reinterpret_cast<FacetSpec*>(pair_smem + RP_PAIR_SPEC_OFF);
    }
    const int tid = threadIdx.x;
    const int nq = A.ntl[s];
    const int n = A.nill[s];
    if (tb * RP_PAIR_THREADS >= nq || n == 0) return true;
    const int nchunks = (n + RP_CHUNK - 1) / RP_CHUNK;
    const int64_t np = (int64_t)1 << lparts;
    const int k0 = (int)((int64_t)nchunks * part / np);
    const int k1 = (int)((int64_t)nchunks * (part + 1) / np);
    if (k0 >= k1) return true;
    const int q = tb * RP_PAIR_THREADS + tid;
    const bool active = q < nq;
    float tnx = 0, tny = 0, tnz = 1;
    int b0 = 0;
    C32* Trow = nullptr;
    C32* Trow2 = nullptr;
    if (active) {
        const int64_t ti = A.tlist[(size_t)s * A.tstride + q];
        // t' = target - trace origin and |t'|^2 (FP64, once per item), kept
        // as double-floats: high parts in s_tq[0], low parts in s_tq[1]
        const double px = A.TG[ti] - A.org[4 * s], py = A.TG[A.nt + ti] - A.org[4 * s + 1],
                     pz = A.TG[2 * A.nt + ti] - A.org[4 * s + 2];
        const double p2 = px * px + py * py + pz * pz;
        const float hx = (float)px, hy = (float)py, hz = (float)pz, h2 = (float)p2;
        s_tq[tid] = make_float4(hx, hy, hz, h2);
        s_tq[RP_PAIR_THREADS + tid] = make_float4((float)(px - hx), (float)(py - hy), (float)(pz - hz),
                                                  (float)(p2 - h2));
        tnx = (float)A.TG[3 * A.nt + ti]; tny = (float)A.TG[4 * A.nt + ti];
        tnz = (float)A.TG[5 * A.nt + ti];
        b0 = A.bt0[(size_t)s * A.tstride + q];
        Trow = A.T + 2 * ((((size_t)part * A.nb + s) * A.tstride + q) * A.Wt);
        if constexpr (SPEC) Trow2 = A.T2 + 2 * ((((size_t)part * A.nb + s) * A.tstride + q) * A.Wt);
    }
    const FacetPair* rbase = A.rec + (size_t)s * (A.rstride / 2);
    const ChunkMeta* mbase = A.meta + (size_t)s * A.mstride;
    // prologue: stage chunk k0 and its metadata (whole pairs: an odd count
    // ends with a padded pair)
    if (tid == 0 && !A.stall_copies) {
        int cnt = min(RP_CHUNK, n - k0 * RP_CHUNK);
        uint32_t bytes = (uint32_t)(((cnt + 1) >> 1) * sizeof(FacetPair));
        const uint32_t sbytes = SPEC ? (uint32_t)(((cnt + 1) >> 1) * sizeof(FacetSpec)) : 0u;
        mbar_expect_tx(&bars[0], bytes + sbytes + (uint32_t)sizeof(ChunkMeta));
        tma_bulk_g2s(srec, rbase + (size_t)k0 * RP_CHUNK_PAIRS, bytes, &bars[0]);
        tma_bulk_g2s(smeta, mbase + k0, (uint32_t)sizeof(ChunkMeta), &bars[0]);
        if constexpr (SPEC)
            tma_bulk_g2s(sspec, A.spec + (size_t)s * (A.rstride / 2) + (size_t)k0 * RP_CHUNK_PAIRS, sbytes, &bars[0]);
    }
    for (int k = k0; k < k1; ++k) {
        const int buf = (k - k0) & 1;
        // prefetch the next chunk into the other buffer (its readers
        // finished at the trailing __syncthreads of the previous step)
        if (tid == 0 && k + 1 < k1 && !A.stall_copies) {
            int cnt = min(RP_CHUNK, n - (k + 1) * RP_CHUNK);
            uint32_t bytes = (uint32_t)(((cnt + 1) >> 1) * sizeof(FacetPair));
            const uint32_t sbytes = SPEC ? (uint32_t)(((cnt + 1) >> 1) * sizeof(FacetSpec)) : 0u;
            mbar_expect_tx(&bars[buf ^ 1], bytes + sbytes + (uint32_t)sizeof(ChunkMeta));
            tma_bulk_g2s(srec + (buf ^ 1) * RP_CHUNK_PAIRS, rbase + (size_t)(k + 1) * RP_CHUNK_PAIRS, bytes,
                         &bars[buf ^ 1]);
            tma_bulk_g2s(smeta + (buf ^ 1), mbase + k + 1, (uint32_t)sizeof(ChunkMeta), &bars[buf ^ 1]);
            if constexpr (SPEC)
                tma_bulk_g2s(sspec + (buf ^ 1) * RP_CHUNK_PAIRS,
                             A.spec + (size_t)s * (A.rstride / 2) + (size_t)(k + 1) * RP_CHUNK_PAIRS, sbytes,
                             &bars[buf ^ 1]);
        }
        const ChunkMeta* mp = smeta + buf;
        const bool got = mbar_wait(&bars[buf], phase[buf], A.spin_limit);
        const bool live = active && got;
        const FacetPair* R = srec + buf * RP_CHUNK_PAIRS;
        const FacetSpec* RS = SPEC ? sspec + buf * RP_CHUNK_PAIRS : nullptr;
        Anchor an;
        int blo = 0;
        bool fits = true;
        if (live) {
            // anchors of this (chunk, target) in double-float FP32
            const float4 th = s_tq[tid], tl = s_tq[RP_PAIR_THREADS + tid];
            const float cfx = mp->cfx, cfy = mp->cfy, cfz = mp->cfz;
            float Th, Tl, Qh;
            anchor_distance(th, tl, cfx, cfy, cfz, mp->cch, mp->ccl, Th, Tl, Qh);
            // n T0 / lam (turns) -> phase; n T0 / dr (bins) -> integer and fraction
            const float fr = frac_dd(Th, Tl, A.kth, A.ktl);
            float xf;
            const int xi = floor_dd(Th, Tl, A.kbh, A.kbl, xf);
            const float lo = xf + mp->lo_off, hi = xf + mp->hi_off;
            const int blo_rel = floor_i(lo) - 1;
            blo = xi + blo_rel;
            // every pair's bin x lies in [lo, hi] (relative to xi; triangle
            // inequality on the chunk's bounding radius); with half a bin of
            // margin for FP32 rounding both split bins stay inside the window
            // and the trace
            fits = blo >= 0 && blo + W <= A.nr1 && hi + 0.5f < (float)(blo_rel + W - 1) &&
                   mp->phase_ok;
            an.Dx = __fadd_rn(__fadd_rn(th.x, -cfx), tl.x);
            an.Dy = __fadd_rn(__fadd_rn(th.y, -cfy), tl.y);
            an.Dz = __fadd_rn(__fadd_rn(th.z, -cfz), tl.z);
            an.T0 = Th; an.T0sq = Qh;
            an.ph0 = -6.28318530717958647f * fr;
            an.xbase = xf - (float)blo_rel;
            an.tnx = tnx; an.tny = tny; an.tnz = tnz;
            an.nDtn = -fmaf(an.Dx, tnx, fmaf(an.Dy, tny, an.Dz * tnz));
            an.eaT0 = fmaf(A.ealpha, Th, A.eks);
        }
        const bool all_fit = __all_sync(0xffffffffu, fits);
        if (live) {
            for (int w = 0; w < W; ++w) win[w * RP_PAIR_THREADS + tid] = make_float2(0.f, 0.f);
            if constexpr (SPEC)
                for (int w = 0; w < W; ++w) win2[w * RP_PAIR_THREADS + tid] = make_float2(0.f, 0.f);
            const int cnt = min(RP_CHUNK, n - k * RP_CHUNK);    // = mp->n (bounds from the count, not the staged copy)
            const int npairs = (cnt + 1) >> 1;
            const bool prisms = (A.np > 0) && !A.lossless;
            int jp = 0;
            if constexpr (SPEC) {
                if (all_fit && !prisms) {
                    for (; jp + ILP <= npairs; jp += ILP) {
                        f2 x[ILP], re[ILP], im[ILP], ga[ILP], gb[ILP];
#pragma unroll
                        for (int i = 0; i < ILP; ++i)
                            pair_eval2s<NT, false>(R[jp + i], RS[jp + i], an, A, x[i], re[i], im[i], ga[i], gb[i]);
#pragma unroll
                        for (int i = 0; i < ILP; ++i) bin_add_fast2s(x[i], re[i], im[i], ga[i], gb[i], win, win2, tid);
                    }
                    for (; jp < npairs; ++jp) {
                        f2 x0, re0, im0, ga, gb;
                        pair_eval2s<NT, false>(R[jp], RS[jp], an, A, x0, re0, im0, ga, gb);
                        bin_add_fast2s(x0, re0, im0, ga, gb, win, win2, tid);
                    }
                } else
                for (; jp < npairs; ++jp) {
                    f2 x0, re0, im0, ga, gb;
                    pair_eval2s<NT>(R[jp], RS[jp], an, A, x0, re0, im0, ga, gb);
                    const bool two = 2 * jp + 1 < cnt;
                    if (prisms) {
                        const FacetPair& r0 = R[jp];
                        const f2 dx = fld<F_DX>(r0), dy = fld<F_DY>(r0), dz = fld<F_DZ>(r0), q = fld<F_Q>(r0);
                        const float f0 = prism_factor(make_float4(dx.x, dy.x, dz.x, q.x), mp->cx, mp->cy, mp->cz,
                                                      an.Dx, an.Dy, an.Dz, an.T0sq, A.PR, A.np, A.ealpha);
                        const float f1 = two ? prism_factor(make_float4(dx.y, dy.y, dz.y, q.y), mp->cx, mp->cy,
                                                            mp->cz, an.Dx, an.Dy, an.Dz, an.T0sq, A.PR, A.np,
                                                            A.ealpha)
                                             : 0.f;
                        re0.x *= f0; im0.x *= f0; re0.y *= f1; im0.y *= f1;
                    }
                    bin_add<W>(x0.x, re0.x * ga.x, im0.x * ga.x, blo, b0, win, tid, Trow, A);
                    bin_add<W>(x0.x, re0.x * gb.x, im0.x * gb.x, blo, b0, win2, tid, Trow2, A);
                    if (two) {
                        bin_add<W>(x0.y, re0.y * ga.y, im0.y * ga.y, blo, b0, win, tid, Trow, A);
                        bin_add<W>(x0.y, re0.y * gb.y, im0.y * gb.y, blo, b0, win2, tid, Trow2, A);
                    }
                }
            } else if (all_fit && !prisms) {
                // ILP pairs per step; binned in facet order, so every ILP
                // gives the same sums
                if (ILP > 1)
                for (; jp + ILP <= npairs; jp += ILP) {
                    f2 x[ILP], am[ILP], cs[ILP], sn[ILP];
#pragma unroll
                    for (int i = 0; i < ILP; ++i) {
                        const FacetPair r0 = R[jp + i];
                        pair_eval2_core<NT, ORTHO, false>(r0, an, A, x[i], am[i], cs[i], sn[i]);
                    }
#pragma unroll
                    for (int i = 0; i < ILP; ++i) bin_add_fast2a<W>(x[i], am[i], cs[i], sn[i], win, tid);
                }
                for (; jp < npairs; ++jp) {
                    const FacetPair r0 = R[jp];
                    f2 x0, am0, cs0, sn0;
                    pair_eval2_core<NT, ORTHO, false>(r0, an, A, x0, am0, cs0, sn0);
                    bin_add_fast2a<W>(x0, am0, cs0, sn0, win, tid);
                }
            } else {
                for (; jp < npairs; ++jp) {
                    const FacetPair r0 = R[jp];
                    f2 x0, re0, im0;
                    pair_eval2<NT, ORTHO>(r0, an, A, x0, re0, im0);
                    const bool two = 2 * jp + 1 < cnt;      // the second facet is not padding
                    if (prisms) {
                        const f2 dx = fld<F_DX>(r0), dy = fld<F_DY>(r0), dz = fld<F_DZ>(r0), q = fld<F_Q>(r0);
                        const float f0 = prism_factor(make_float4(dx.x, dy.x, dz.x, q.x), mp->cx, mp->cy, mp->cz,
                                                      an.Dx, an.Dy, an.Dz, an.T0sq, A.PR, A.np, A.ealpha);
                        const float f1 = two ? prism_factor(make_float4(dx.y, dy.y, dz.y, q.y), mp->cx, mp->cy,
                                                            mp->cz, an.Dx, an.Dy, an.Dz, an.T0sq, A.PR, A.np,
                                                            A.ealpha)
                                             : 0.f;
                        re0.x *= f0; im0.x *= f0; re0.y *= f1; im0.y *= f1;
                    }
                    bin_add<W>(x0.x, re0.x, im0.x, blo, b0, win, tid, Trow, A);
                    if (two) bin_add<W>(x0.y, re0.y, im0.y, blo, b0, win, tid, Trow, A);
                }
            }
            // flush the window into the owned trace (both legs' in specular mode)
            flush_window<W>(win, tid, blo, b0, Trow, A.Wt, A.err);
            if constexpr (SPEC) flush_window<W>(win2, tid, blo, b0, Trow2, A.Wt, A.err);
        }
        // everyone done with buffer `buf` before it is refilled; a wait that
        // ran out anywhere in the block ends its work
        if (__syncthreads_or(!got)) {
            abort_block(A, bars, phase, buf, got, k + 1 < k1);
            return false;
        }
        phase[buf] ^= 1u;
    }
    return true;
}

// --------------------------------------------------- ttype-0 targets --
// Two (facet, target) evaluations for a ttype-0 target: genRefrPhasor
// (radar_kernels.cu:351-398) with compRefrEnergyIn/Out's factors
// (geometry_kernels.cu:520-584).  Amplitude rerad(TargetTh) fEI fEO
// radarEq(Itd + Ttd), phase +4 pi_F rngt / lam, bin (rngt - rst) / dr at
// rngt = Itd + Ttd c1/c2.  fEI fEO = att^2 rough^2 frc^2 (times both
// reradiation factors in specular mode), and att^2 rough^2 = exp2(4 e2) with
// pair_eval2's exponent e2; frc^2 and the radar equation's constants are the
// record's a0.  The facet's part of the phase, 4 pi_F Itd / lam, is -2 times
// the record's -2 pi frac(Itd / lam_F) (mod 2 pi).
template <int NT, bool ORTHO, bool SPEC>
__device__ __forceinline__ void pair_eval2t0(const FacetPair& r, const FacetSpec* sp, const FacetT0& t0,
                                             const Anchor& an, const PairArgs& A, f2& xr, f2& vre, f2& vim) {
    const f2 ONE = bc(1.f);
    const f2 dx = fld<F_DX>(r), dy = fld<F_DY>(r), dz = fld<F_DZ>(r);
    const f2 mx = bc(-2.f * an.Dx), my = bc(-2.f * an.Dy), mz = bc(-2.f * an.Dz);
    const f2 qd = fma2(mx, dx, fma2(my, dy, fma2(mz, dz, fld<F_Q>(r))));   // Ttd^2 - T0^2
    const f2 d2 = add2(bc(an.T0sq), qd);
    const f2 rinv = make_float2(rsqrt_a(d2.x), rsqrt_a(d2.y));
    const f2 sT = fma2(d2, rinv, bc(an.T0));
    const f2 dT = mul2(qd, make_float2(rcp_a(sT.x), rcp_a(sT.y)));
    f2 aT, ptr, gg = ONE;
    if (ORTHO) {
        const f2 pc = fma2(mx, fld<F_UX>(r), fma2(my, fld<F_UY>(r), fma2(mz, fld<F_UZ>(r), fld<F_AU>(r))));
        const f2 pd = fma2(mx, fld<F_VX>(r), fma2(my, fld<F_VY>(r), fma2(mz, fld<F_VZ>(r), fld<F_AV>(r))));
        const f2 pt = fma2(dx, bc(an.tnx), fma2(dy, bc(an.tny), fma2(dz, bc(an.tnz), bc(an.nDtn))));
        const f2 pcr = mul2(pc, rinv), pdr = mul2(pd, rinv);
        ptr = mul2(pt, rinv);
        aT = fma2(pdr, pdr, mul2(pcr, pcr));
    } else {
        const f2 hf = bc(0.5f);
        const f2 ex = fma2(mx, hf, dx), ey = fma2(my, hf, dy), ez = fma2(mz, hf, dz);
        const f2 pb = fma2(ex, fld<F_NX>(r), fma2(ey, fld<F_NY>(r), mul2(ez, fld<F_NZ>(r))));
        const f2 pt = fma2(ex, bc(an.tnx), fma2(ey, bc(an.tny), mul2(ez, bc(an.tnz))));
        const f2 pbr = mul2(pb, rinv);
        ptr = mul2(pt, rinv);
        aT = fma2(pbr, neg2(pbr), ONE);
        if (SPEC) {
            const f2 pc = fma2(ex, fld<F_UX>(r), fma2(ey, fld<F_UY>(r), mul2(ez, fld<F_UZ>(r))));
            const f2 pd = add2(fma2(ex, fld<F_VX>(r), fma2(ey, fld<F_VY>(r), mul2(ez, fld<F_VZ>(r)))),
                               bc(-1e-15f));
            const f2 h2 = fma2(pc, pc, mul2(pd, pd));
            const f2 rh = make_float2(rcp_a(h2.x), rcp_a(h2.y));
            f2 g1, g2;
            spec_rerad2<NT>(*sp, A, pbr, aT, pc, pd, rh, g1, g2);
            const f2 g = mul2(g1, g2);
            gg = mul2(g, g);
        }
    }
    // rerad_funct of TargetTh (radar_kernels.cu:167-189): cos TargetTh = ptr
    f2 rr = ONE;
    if (A.rf >= 1 && A.rf <= 3) {
        rr = make_float2(ptr.x > A.rcos ? 1.f : 0.f, ptr.y > A.rcos ? 1.f : 0.f);
    } else if (A.rf == 4) {
        const float th0 = acosf(fminf(1.f, fmaxf(-1.f, ptr.x))), th1 = acosf(fminf(1.f, fmaxf(-1.f, ptr.y)));
        rr = make_float2(ex2_a(A.rgl * th0 * th0), ex2_a(A.rgl * th1 * th1));
    }
    const f2 e2 = fma2(bc(-A.eks), aT, fma2(bc(A.ealpha), dT, bc(an.eaT0)));
    const f2 e4 = mul2(e2, bc(4.f));
    // radarEq: a0 / (Itd + Ttd)^4
    const f2 fS = add2(make_float2(t0.v.z, t0.v.w), add2(bc(an.T0), dT));
    const f2 ri = make_float2(rcp_a(fS.x), rcp_a(fS.y));
    const f2 r2 = mul2(ri, ri);
    const f2 amp = mul2(mul2(mul2(make_float2(t0.v.x, t0.v.y), mul2(r2, r2)), mul2(rr, gg)),
                        make_float2(ex2_a(e4.x), ex2_a(e4.y)));
    f2 ph = fma2(bc(A.kr0), dT, fma2(fld<F_PH>(r), bc(-2.f), bc(an.ph0)));
    const f2 k = mul2(ph, bc(0.159154943091895336f));
    ph = fma2(make_float2(rintf(k.x), rintf(k.y)), bc(-6.28318530717958647f), ph);
    f2 sn, cs;
    __sincosf(ph.x, &sn.x, &cs.x);
    __sincosf(ph.y, &sn.y, &cs.y);
    vre = mul2(amp, cs);
    vim = mul2(amp, sn);
    xr = fma2(bc(A.kb0), dT, add2(fld<F_XI>(r), bc(an.xbase)));
}

// Shared memory of the ttype-0 pair kernel: pair_item's layout, then the
// staged FacetT0 and (specular) FacetSpec chunks.
__host__ __device__ constexpr size_t pair_t0_off(int W) { return pair_smem_bytes(W); }
__host__ __device__ constexpr size_t pair_t0spec_off(int W) { return pair_t0_off(W) + 2 * RP_CHUNK_PAIRS * sizeof(FacetT0); }
__host__ __device__ constexpr size_t pair_t0_smem_bytes(int W, bool spec) {
    return pair_t0spec_off(W) + (spec ? 2 * RP_CHUNK_PAIRS * sizeof(FacetSpec) : 0);
}
static_assert(pair_t0spec_off(RP_WIN_WIDE) % 16 == 0, "staged by bulk copies");

// One work item of the ttype-0 pair kernel: the targets [tq0[s], ntl[s]) of
// trace s, block tb of them, facet-range part `part`.  The chunk staging and
// the double-float anchors are pair_item's; the anchors use c1/c2 in place
// of n and a positive phase, and every phasor goes to one bin.
template <int NT, int ILP, bool ORTHO, bool SPEC, int W>
__device__ __forceinline__ bool pair_item_t0(const PairArgs& A, int s, int tb, int part, uint64_t* bars,
                                             uint32_t* phase) {
    FacetPair* srec = reinterpret_cast<FacetPair*>(pair_smem);
    float2* win = reinterpret_cast<float2*>(pair_smem + pair_win_off());
    float4* s_tq = reinterpret_cast<float4*>(pair_smem + pair_tpos_off(W));
    ChunkMeta* smeta = reinterpret_cast<ChunkMeta*>(pair_smem + pair_meta_off(W));
    FacetT0* st0 = reinterpret_cast<FacetT0*>(pair_smem + pair_t0_off(W));
    FacetSpec* sspec = SPEC ? reinterpret_cast<FacetSpec*>(pair_smem + pair_t0spec_off(W)) : nullptr;
    const int tid = threadIdx.x;
    const int qs = A.tq0[s];
    const int nq = A.ntl[s] - qs;
    const int n = A.nill[s];
    if (tb * RP_PAIR_THREADS >= nq || n == 0) return true;
    const int nchunks = (n + RP_CHUNK - 1) / RP_CHUNK;
    const int k0 = (int)((int64_t)nchunks * part / RP_PARTS);
    const int k1 = (int)((int64_t)nchunks * (part + 1) / RP_PARTS);
    if (k0 >= k1) return true;
    const int ql = tb * RP_PAIR_THREADS + tid;
    const bool active = ql < nq;
    const int q = qs + ql;
    float tnx = 0, tny = 0, tnz = 1;
    int b0 = 0;
    C32* Trow = nullptr;
    if (active) {
        const int64_t ti = A.tlist[(size_t)s * A.tstride + q];
        const double px = A.TG[ti] - A.org[4 * s], py = A.TG[A.nt + ti] - A.org[4 * s + 1],
                     pz = A.TG[2 * A.nt + ti] - A.org[4 * s + 2];
        const double p2 = px * px + py * py + pz * pz;
        const float hx = (float)px, hy = (float)py, hz = (float)pz, h2 = (float)p2;
        s_tq[tid] = make_float4(hx, hy, hz, h2);
        s_tq[RP_PAIR_THREADS + tid] = make_float4((float)(px - hx), (float)(py - hy), (float)(pz - hz),
                                                  (float)(p2 - h2));
        tnx = (float)A.TG[3 * A.nt + ti]; tny = (float)A.TG[4 * A.nt + ti];
        tnz = (float)A.TG[5 * A.nt + ti];
        b0 = A.bt0[(size_t)s * A.tstride + q];
        Trow = A.T + 2 * ((((size_t)part * A.nb + s) * A.tstride + q) * A.Wt);
    }
    const size_t pbase = (size_t)s * (A.rstride / 2);
    const FacetPair* rbase = A.rec + pbase;
    const ChunkMeta* mbase = A.meta + (size_t)s * A.mstride;
    auto stage = [&](int k, int b) {
        const int cnt = min(RP_CHUNK, n - k * RP_CHUNK);
        const uint32_t np = (uint32_t)((cnt + 1) >> 1);
        const uint32_t bytes = np * (uint32_t)sizeof(FacetPair), tb0 = np * (uint32_t)sizeof(FacetT0);
        const uint32_t sb = SPEC ? np * (uint32_t)sizeof(FacetSpec) : 0u;
        mbar_expect_tx(&bars[b], bytes + tb0 + sb + (uint32_t)sizeof(ChunkMeta));
        tma_bulk_g2s(srec + b * RP_CHUNK_PAIRS, rbase + (size_t)k * RP_CHUNK_PAIRS, bytes, &bars[b]);
        tma_bulk_g2s(smeta + b, mbase + k, (uint32_t)sizeof(ChunkMeta), &bars[b]);
        tma_bulk_g2s(st0 + b * RP_CHUNK_PAIRS, A.t0rec + pbase + (size_t)k * RP_CHUNK_PAIRS, tb0, &bars[b]);
        if (SPEC)
            tma_bulk_g2s(sspec + b * RP_CHUNK_PAIRS, A.spec + pbase + (size_t)k * RP_CHUNK_PAIRS, sb, &bars[b]);
    };
    if (tid == 0 && !A.stall_copies) stage(k0, 0);
    for (int k = k0; k < k1; ++k) {
        const int buf = (k - k0) & 1;
        if (tid == 0 && k + 1 < k1 && !A.stall_copies) stage(k + 1, buf ^ 1);
        const ChunkMeta* mp = smeta + buf;
        const bool got = mbar_wait(&bars[buf], phase[buf], A.spin_limit);
        const bool live = active && got;
        const FacetPair* R = srec + buf * RP_CHUNK_PAIRS;
        const FacetT0* R0 = st0 + buf * RP_CHUNK_PAIRS;
        const FacetSpec* RS = SPEC ? sspec + buf * RP_CHUNK_PAIRS : nullptr;
        Anchor an;
        int blo = 0;
        bool fits = true;
        if (live) {
            const float4 th = s_tq[tid], tl = s_tq[RP_PAIR_THREADS + tid];
            const float cfx = mp->cfx, cfy = mp->cfy, cfz = mp->cfz;
            float Th, Tl, Qh;
            anchor_distance(th, tl, cfx, cfy, cfz, mp->cch, mp->ccl, Th, Tl, Qh);
            const float fr = frac_dd(Th, Tl, A.kt0h, A.kt0l);
            float xf;
            const int xi = floor_dd(Th, Tl, A.kb0h, A.kb0l, xf);
            const float lo = xf + fmaf(-A.kb0, mp->R, mp->xmin), hi = xf + fmaf(A.kb0, mp->R, mp->xmax);
            const int blo_rel = floor_i(lo) - 1;
            blo = xi + blo_rel;
            fits = blo >= 0 && blo + W <= A.nr && hi + 0.5f < (float)(blo_rel + W);
            an.Dx = __fadd_rn(__fadd_rn(th.x, -cfx), tl.x);
            an.Dy = __fadd_rn(__fadd_rn(th.y, -cfy), tl.y);
            an.Dz = __fadd_rn(__fadd_rn(th.z, -cfz), tl.z);
            an.T0 = Th; an.T0sq = Qh;
            an.ph0 = 6.28318530717958647f * fr;
            an.xbase = xf - (float)blo_rel;
            an.tnx = tnx; an.tny = tny; an.tnz = tnz;
            an.nDtn = -fmaf(an.Dx, tnx, fmaf(an.Dy, tny, an.Dz * tnz));
            an.eaT0 = fmaf(A.ealpha, Th, A.eks);
        }
        const bool all_fit = __all_sync(0xffffffffu, fits);
        if (live) {
            for (int w = 0; w < W; ++w) win[w * RP_PAIR_THREADS + tid] = make_float2(0.f, 0.f);
            const int cnt = min(RP_CHUNK, n - k * RP_CHUNK);
            const int npairs = (cnt + 1) >> 1;
            const bool prisms = A.np > 0;
            int jp = 0;
            if (all_fit && !prisms) {
                // every pair's bin is inside the window and the trace
                for (; jp < npairs; jp += ILP) {
                    f2 x[ILP], re[ILP], im[ILP];
#pragma unroll
                    for (int i = 0; i < ILP; ++i) {
                        const int j = min(jp + i, npairs - 1);
                        pair_eval2t0<NT, ORTHO, SPEC>(R[j], SPEC ? RS + j : nullptr, R0[j], an, A, x[i], re[i], im[i]);
                    }
#pragma unroll
                    for (int i = 0; i < ILP; ++i) {
                        if (jp + i >= npairs) break;
                        const unsigned s0 = min((unsigned)floor_i(x[i].x), (unsigned)(W - 1));
                        const unsigned s1 = min((unsigned)floor_i(x[i].y), (unsigned)(W - 1));
                        float2* p0 = &win[s0 * RP_PAIR_THREADS + tid];
                        float2 v0 = *p0;
                        v0.x += re[i].x;
                        v0.y += im[i].x;
                        *p0 = v0;
                        float2* p1 = &win[s1 * RP_PAIR_THREADS + tid];
                        float2 v1 = *p1;
                        v1.x += re[i].y;
                        v1.y += im[i].y;
                        *p1 = v1;
                    }
                }
            } else {
                for (; jp < npairs; ++jp) {
                    f2 x0, re0, im0;
                    pair_eval2t0<NT, ORTHO, SPEC>(R[jp], SPEC ? RS + jp : nullptr, R0[jp], an, A, x0, re0, im0);
                    const bool two = 2 * jp + 1 < cnt;
                    if (prisms) {
                        // the prisms' change of att, squared (att^2 here, sqrt(att) in prism_factor);
                        // ttype-0 targets take fEI and fEO whatever lossless says (sim.cu:940-966)
                        const FacetPair& r0 = R[jp];
                        const f2 dx = fld<F_DX>(r0), dy = fld<F_DY>(r0), dz = fld<F_DZ>(r0), qq = fld<F_Q>(r0);
                        float f0 = prism_factor(make_float4(dx.x, dy.x, dz.x, qq.x), mp->cx, mp->cy, mp->cz,
                                                an.Dx, an.Dy, an.Dz, an.T0sq, A.PR, A.np, A.ealpha);
                        float f1 = two ? prism_factor(make_float4(dx.y, dy.y, dz.y, qq.y), mp->cx, mp->cy, mp->cz,
                                                      an.Dx, an.Dy, an.Dz, an.T0sq, A.PR, A.np, A.ealpha)
                                       : 0.f;
                        f0 *= f0; f0 *= f0; f1 *= f1; f1 *= f1;
                        re0.x *= f0; im0.x *= f0; re0.y *= f1; im0.y *= f1;
                    }
                    bin_add1<W>(x0.x, re0.x, im0.x, blo, b0, win, tid, Trow, A);
                    if (two) bin_add1<W>(x0.y, re0.y, im0.y, blo, b0, win, tid, Trow, A);
                }
            }
            flush_window<W>(win, tid, blo, b0, Trow, A.Wt, A.err);
        }
        if (__syncthreads_or(!got)) {
            abort_block(A, bars, phase, buf, got, k + 1 < k1);
            return false;
        }
        phase[buf] ^= 1u;
    }
    return true;
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

// Launches of the per-kind multi-job kernels k_pairs32mk (rp_multi.cu), one
// per (sinc degree, frame kind) group of h_jobs (host copies); work[j] is
// job j's counter; cfg 0: 3 facet pairs per step, 1: 4.  With naux > 0 the
// launches go round robin to the streams aux[0 .. naux), so the groups run
// concurrently and one group's tail is filled by another's blocks (the
// caller forks those streams from its own and joins them back); else all
// on st.
int launch_pairs_multik(int cfg, const PairJob* h_jobs, int njobs, unsigned int* work, int sms, cudaStream_t st,
                        const cudaStream_t* aux = nullptr, int naux = 0);

// Launch of the specular-mode pair kernel k_pairs32s (rp_spec.cu) of sinc
// degree deg in configuration cfg (0 or 1) over items work items.
int launch_pairs_spec(int deg, int cfg, const PairArgs& P, int64_t items, int sms, cudaStream_t st);

// Launch of the ttype-0 pair kernel k_pairs32t0 (rp_spec.cu) over items work
// items (deg matters in specular mode only).
int launch_pairs_t0(int deg, bool ortho, bool spec, const PairArgs& P, int64_t items, int sms, cudaStream_t st);

// Specular mode without convolution (rp_direct.cu): the direct sums of
// reflRadarSignal and refrRadarSignal per (trace, bin).
#define RP_DS_THREADS 256     // facets per staged chunk
#define RP_DS_BPT 8           // bins per thread (strided by RP_DS_THREADS)
#define RP_DS_TILE (RP_DS_THREADS * RP_DS_BPT)
#define RP_DS_GROUPS 128      // fixed facet-chunk groups per trace (ordered partial sums)
struct DirectArgs {
    const double* F;        // sorted facet store, SoA [12][nf]
    int64_t nf;             // its stride
    int64_t fstride;        // per-trace stride of idx and sv (the segment's facet capacity)
    const int* idx;         // [nb][fstride] illuminated facets (store order)
    const int* nill;
    const double* traces;   // [nb][9]
    const double* TG;       // fast target store [7][nt]
    int64_t nt;
    const int* tlist;       // [nb][tstride] in-aperture targets (all ttype 0 in this mode)
    const int* ntl;
    int64_t tstride;
    const C32* sv;          // [nb][fstride] surface phasors fRe exp(+j 4 pi_F Itd / lam)
    const FacetSpec* spec;  // [nb][rstride / 2]
    const FacetT0* t0rec;   // [nb][rstride / 2]
    int64_t rstride;
    const double* PR;       // prisms
    int64_t np;
    int nr;
    double beta;            // dr / rng_res: sinc((r - R)/res) = sinc(beta (i - x))
    double inv_dr;
    double turn2;           // 2 turn: phase 4 pi_F R / lam = 2 pi (turn2 R)
    double c_c2;            // c / c2 of refrRadarSignal's range
    double alpha2;
    float ks2;              // ks^2
    float e21, s2tir, pikr2;
    int rf;
    float rcos, rgl;
    double2* part;          // [nb][RP_DS_GROUPS][nr]
};
int launch_direct(const DirectArgs& A, int nb, void* d_out, int out64, int s0, cudaStream_t st);

}  // namespace rpk
