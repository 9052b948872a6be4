// rp_fast.cu -- the fused FP32 split-precision form.
//
// Per batch of traces:
//   1. aperture cull + ordered compaction of the spatially (Morton) sorted
//      facet store (rp_common.cuh);
//   2. k_facets32: per (trace, chunk of RP_CHUNK facets) the incident leg in
//      FP64 (compIncidentRays, snellsLaw, compReflectedEnergy, surfacePT) and
//      a 64-byte FP32 record per facet: position relative to the chunk centre,
//      frame vectors, the bin offset (Itd - rst)/dr, the incident phase in
//      turns mod 1, and the hoisted amplitude factor;
//   3. k_pairs32 (the hot kernel): each thread owns one in-aperture target of
//      one trace and walks the trace's chunks, staged in shared memory by a
//      TMA bulk copy.  Per (chunk, target) it forms FP64 anchors (distance,
//      bin and phase of the chunk centre); per (facet, target) pair it
//      evaluates the target leg in FP32 on small differences from those
//      anchors and bins the phasor into a per-thread shared-memory window,
//      flushed to the target's trace after the chunk.  Single ownership makes
//      the accumulation deterministic without atomics;
//   4. k_conv32: per target, range compression (chirp convolution and the
//      cropped, decimated convolveComplex) -- the outbound leg is the inbound
//      leg times -1/sqrt(P) (radiateTarget = accumulateTarget with P = 1 and
//      the phase of rngt - lam/2, radar_kernels.cu:834-892);
//   5. surface range compression and a fixed-order sum over targets.
//
// Specular mode with linear convolution runs the same stages: the surface
// leg is genReflPhasor's one-bin phasor of the specular energy
// (radar_kernels.cu:314-346, geometry_kernels.cu:434-446), the pair kernel
// is k_pairs32s (rp_spec.cu), which bins the outbound leg (with its own
// facetReradiation factor) into a second trace T2, and compression uses T2
// as Psour and the surface chirp for both target legs (specular mode never
// regenerates it, sim.cu:851-856).
#include <algorithm>
#include <climits>
#include <cstring>
#include <cmath>
#include <map>
#include <atomic>
#include <mutex>
#include <thread>
#include <vector>

#include "rp_common.cuh"
#include "rp_conv.cuh"
#include "rp_convs.cuh"
#include "rp_fft.cuh"
#include "rp_pair.cuh"

using namespace rpk;

namespace {

using C64 = Cx<double>;

// --------------------------------------------------------- block reduce --
template <class T, class Op>
__device__ T block_reduce(T v, Op op, T* sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    T r = sh[0];
    for (int w = 1; w < nw; ++w) r = op(r, sh[w]);
    __syncthreads();
    return r;
}

// Block-wide maxima of N floats at once: one shared-memory round and two
// barriers for all of them (sh: N x 32 floats).  Minima are maxima of the
// negated values.
template <int N>
__device__ __forceinline__ void block_max_n(float (&v)[N], float* sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] = fmaxf(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < N; ++k) sh[k * 32 + wid] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; ++k) {
        float r = sh[k * 32];
        for (int w = 1; w < nw; ++w) r = fmaxf(r, sh[k * 32 + w]);
        v[k] = r;
    }
    __syncthreads();
}

struct MinOp { __device__ double operator()(double a, double b) const { return fmin(a, b); } };
struct MaxOp { __device__ double operator()(double a, double b) const { return fmax(a, b); } };
struct MinOpF { __device__ float operator()(float a, float b) const { return fminf(a, b); } };
struct MaxOpF { __device__ float operator()(float a, float b) const { return fmaxf(a, b); } };

// ------------------------------------------------------ per-facet stage --
// Specular mode's surface amplitude (genReflPhasor's fRe): facetReradiation
// at twice the inclination times the radar equation, times rho^2 atm rough
// (fre), geometry_kernels.cu:434-446; sin 2th = 2 sI cI.
__device__ __forceinline__ float spec_surface_amp(const DevParams& dp, double grefl, double d, int n, float sI,
                                                      float cI, float cph, float sph, float fre) {
    const double fl = dp.fs / dp.lam, s2t = 2.0 * (double)sI * (double)cI;
    const double v = (dp.fs * dp.fs / dp.lam) * d_sinc(fl * s2t * (double)cph) * d_sinc(-fl * s2t * (double)sph);
    return (float)(v * v * d_radar_eq(dp.P, grefl, dp.fs, dp.lam, d, (double)n) * (double)fre);
}

// SPEC: specular mode (the scene's dp.specular); T0: the scene has ttype-0
// targets (FacetT0 records).  Separate instantiations, so the default mode's
// kernel carries none of their code.
template <bool SPEC, bool T0>
__global__ void __launch_bounds__(RP_CHUNK)
k_facets32(const double* __restrict__ F, int64_t nf, int64_t fstride, const int* __restrict__ idx,
           const int* __restrict__ nill, const double* __restrict__ traces, DevParams dp,
           FacetPair* __restrict__ rec, ChunkMeta* __restrict__ meta, int64_t rstride,
           int64_t mstride, float* __restrict__ sx_o, C32* __restrict__ sv_o,
           unsigned long long* __restrict__ vmax, double* __restrict__ org,
           const int64_t* __restrict__ order, FacetSpec* __restrict__ spec, FacetT0* __restrict__ t0rec) {
    __shared__ float shf[6 * 32];
    const int s = blockIdx.y;
    const int n = nill[s];
    const int k = blockIdx.x;
    const int j = k * RP_CHUNK + threadIdx.x;
    if (k * RP_CHUNK >= n) return;                  // whole block exits together
    const bool ok = j < n;
    const TraceRow t = load_trace(traces, s);
    double fx = 0, fy = 0, fz = 0;
    int64_t i = 0;
    if (ok) {
        i = idx[(size_t)s * fstride + j];
        fx = F[i]; fy = F[nf + i]; fz = F[2 * nf + i];
    }
    // the trace origin is its first illuminated facet.  The chunk's bounding
    // box comes from the facets' FP32 offsets from the origin (one combined
    // reduction: FP64 minima and maxima would run on the narrow FP64 pipe),
    // widened by the offsets' rounding so that it holds every facet.  The
    // chunk centre is the origin plus the box centre cf, an FP32 offset, so
    // cf is exact in FP32 by construction.
    const int64_t i0 = idx[(size_t)s * fstride];
    const double ox = F[i0], oy = F[nf + i0], oz = F[2 * nf + i0];
    float bx[6];
    {
        const float qx = (float)(fx - ox), qy = (float)(fy - oy), qz = (float)(fz - oz);
        bx[0] = ok ? -qx : -3e38f; bx[1] = ok ? -qy : -3e38f; bx[2] = ok ? -qz : -3e38f;
        bx[3] = ok ? qx : -3e38f; bx[4] = ok ? qy : -3e38f; bx[5] = ok ? qz : -3e38f;
    }
    block_max_n<6>(bx, shf);
    const float qmnx = -bx[0], qmny = -bx[1], qmnz = -bx[2], qmxx = bx[3], qmxy = bx[4], qmxz = bx[5];
    const float cfx = 0.5f * (qmnx + qmxx), cfy = 0.5f * (qmny + qmxy), cfz = 0.5f * (qmnz + qmxz);
    const double cx = ox + (double)cfx, cy = oy + (double)cfy, cz = oz + (double)cfz;
    // |FP32 rounding of an offset q| <= |q| 2^-24: widen by 2^-23 of the extent and 1 micrometre
    auto lo_edge = [](double o, float q) { return o + (double)q - (fabs((double)q) * 0x1p-23 + 1e-6); };
    auto hi_edge = [](double o, float q) { return o + (double)q + (fabs((double)q) * 0x1p-23 + 1e-6); };
    const double mnx = lo_edge(ox, qmnx), mny = lo_edge(oy, qmny), mnz = lo_edge(oz, qmnz);
    const double mxx = hi_edge(ox, qmxx), mxy = hi_edge(oy, qmxy), mxz = hi_edge(oz, qmxz);
    if (k == 0 && threadIdx.x == 0) {
        org[4 * s] = ox; org[4 * s + 1] = oy; org[4 * s + 2] = oz; org[4 * s + 3] = 0.0;
    }
    float xI = 0.f, rr = 0.f, amax = 0.f;
    float spR = 0.f, spC = 1.f, spI = 1.f, spS = 0.f;    // sin/cos Rth, cos/sin Iph (specular records)
    float t0a = 0.f, t0d = 0.f;                          // FacetT0: a0 and Itd
    float fv[RP_NFIELD];            // this facet's record fields (FacetField order)
#pragma unroll
    for (int f = 0; f < RP_NFIELD; ++f) fv[f] = 0.f;
    if (ok) {
        // FP64: the range and everything that becomes a phase or a bin
        // offset; FP32: the angles and amplitudes (relative error ~1e-6).
        // Angles enter only through their cosines and sines, formed from dot
        // and cross products: cos th = -I.n, sin th = |I x n| (accurate near
        // nadir), cos ph / sin ph = (I.v, I.u) / |(I.v, I.u)| (atan2(0, 0) =
        // 0), Snell's cos = sqrt(1 - sR^2) (cos(1e4) on total internal
        // reflection, as the reference's flag value gives).
        const double dxd = fx - t.sx, dyd = fy - t.sy, dzd = fz - t.sz;
        const double d = sqrt(dxd * dxd + dyd * dyd + dzd * dzd);
        const float inv_d = 1.f / (float)d;                 // angles are FP32
        const float Ix = (float)dxd * inv_d, Iy = (float)dyd * inv_d, Iz = (float)dzd * inv_d;
        const double nx = F[3 * nf + i], ny = F[4 * nf + i], nz = F[5 * nf + i];
        const double ux = F[6 * nf + i], uy = F[7 * nf + i], uz = F[8 * nf + i];
        const double vx = F[9 * nf + i], vy = F[10 * nf + i], vz = F[11 * nf + i];
        const float nxf = (float)nx, nyf = (float)ny, nzf = (float)nz;
        const float cI = fminf(1.f, fmaxf(-1.f, -(Ix * nxf + Iy * nyf + Iz * nzf)));
        const float crx = Iy * nzf - Iz * nyf, cry = Iz * nxf - Ix * nzf, crz = Ix * nyf - Iy * nxf;
        const float sI = fminf(1.f, sqrtf(crx * crx + cry * cry + crz * crz));
        const float pu = Ix * (float)ux + Iy * (float)uy + Iz * (float)uz;
        const float pv = Ix * (float)vx + Iy * (float)vy + Iz * (float)vz;
        const float hh = sqrtf(pu * pu + pv * pv);
        const float cph = hh > 0.f ? pv / hh : 1.f, sph = hh > 0.f ? pu / hh : 0.f;
        const float sR = (float)dp.sqrt_eps12 * sI;
        const bool tir = sR > 1.f;
        const float cR = tir ? cosf(1e4f) : sqrtf(fmaxf(0.f, 1.f - sR * sR));
        const float nu1 = (float)dp.nu1, nu2 = (float)dp.nu2;
        const float rho = (nu2 * cI - nu1 * cR) / (nu2 * cI + nu1 * cR);
        const float df = (float)d;
        const float atm = expf(-4.0f * (float)dp.alpha1 * df);
        const float frc = tir ? 0.f : (1.f - rho * rho) * atm;
        const float ksc = (float)dp.ks * cI;
        const float fre = rho * rho * atm * expf(-4.f * ksc * ksc);
        // facet_G (radar_kernels.cu:658-677), sinc(x) = sin(pi x)/(pi x)
        const float lamf = (float)dp.lam, fsf = (float)dp.fs;
        const float piLlam = (float)RP_PI_F * fsf / lamf;
        const float a1 = (float)RP_PI * piLlam * sI * cph, a2 = (float)RP_PI * piLlam * sI * sph;
        const float s1 = fabsf(a1) < 3.14159265e-6f ? 1.f : sinf(a1) / a1;
        const float s2 = fabsf(a2) < 3.14159265e-6f ? 1.f : sinf(a2) / a2;
        const float D = (s1 * s2) * (s1 * s2);
        const float G = D * (4.f * (float)RP_PI_F * fsf * fsf) / (lamf * lamf);
        const float f4 = (4.f * (float)RP_PI_FRIIS) * (4.f * (float)RP_PI_FRIIS);
        const float grefr = (float)t.grefr;
        // phase in turns: phasor(2 Itd) = exp(-j (2 pi_F/lam) 2 Itd) = exp(-j 2 pi tt)
        const double tt = 2.0 * d * dp.turn;
        const float ft = (float)(tt - floor(tt));
        float sn, cs, amp;
        if constexpr (SPEC) {
            // genReflPhasor: fRe exp(+j 4 pi_F Itd / lam)
            amp = spec_surface_amp(dp, t.grefl, d, n, sI, cI, cph, sph, fre);
            sincospif(2.f * ft, &sn, &cs);
            spR = tir ? sinf(1e4f) : sR;
            spC = cR;
            spI = cph;
            spS = sph;
        } else {
            // surface leg (surfacePT, radar_kernels.cu:714-764): two Friis hops
            const float hop = lamf * lamf * G * grefr / (f4 * df * df);
            float Ps = (float)dp.P * hop * hop;
            if (!dp.lossless) Ps *= fre;
            amp = sqrtf(Ps);
            if (dp.incoherent)      // randomPhasor (radar_kernels.cu:741-742), seeded by the facet's input index
                sincospif(2.f * (float)rp_incoherent_turns(dp.inc_seed, t.sx, t.sy, t.sz, order[i]), &sn, &cs);
            else
                sincospif(-2.f * ft, &sn, &cs);
        }
        xI = (float)((d - t.rst) * dp.inv_dr);
        sx_o[(size_t)s * fstride + j] = xI;
        sv_o[(size_t)s * fstride + j] = C32{amp * cs, amp * sn};
        amax = fabsf(amp);
        // hoisted target-leg amplitude: sqrt(P Gr G frc n) lam^2 Dmax / ((4 pi)^2 Itd),
        // times fs^2 / lam of the reradiation factors in specular mode
        const float Dmax = (4.f * (float)RP_PI_F * fsf * fsf) / (lamf * lamf);
        const float Kf = sqrtf((float)dp.P * grefr * G * (dp.lossless ? 1.f : frc) * (float)dp.nidx) * lamf *
                         lamf * Dmax / (f4 * df) * ((SPEC && !dp.lossless) ? (float)(dp.fs * dp.fs / dp.lam) : 1.f);
        if constexpr (T0) {
            // genRefrPhasor's per-facet constants: frc^2 (fEI fEO) and radarEq's
            // nill P Grefr^2 fs^4 / (4 pi)^2, times (fs^2/lam)^4 of the two
            // reradiation factors in specular mode
            const double f4d = (4.0 * RP_PI_FRIIS) * (4.0 * RP_PI_FRIIS), fs2 = dp.fs * dp.fs;
            double a0 = (double)frc * (double)frc * (double)n * dp.P * t.grefr * t.grefr * fs2 * fs2 / f4d;
            if (SPEC) {
                const double r = fs2 / dp.lam;
                a0 *= (r * r) * (r * r);
            }
            t0a = (float)a0;
            t0d = (float)d;
        }
        const double ti = d * dp.turn;
        float ddx = (float)(fx - cx), ddy = (float)(fy - cy), ddz = (float)(fz - cz);
        rr = sqrtf(ddx * ddx + ddy * ddy + ddz * ddz);
        fv[F_DX] = ddx; fv[F_DY] = ddy; fv[F_DZ] = ddz; fv[F_Q] = ddx * ddx + ddy * ddy + ddz * ddz;
        if (dp.ortho) {         // a.u and a.v in place of the normal (exact products, one rounding)
            fv[F_AU] = (float)((double)ddx * (float)ux + (double)ddy * (float)uy + (double)ddz * (float)uz);
            fv[F_AV] = (float)((double)ddx * (float)vx + (double)ddy * (float)vy + (double)ddz * (float)vz);
            fv[F_NZ] = 0.f;
        } else {
            fv[F_NX] = (float)nx; fv[F_NY] = (float)ny; fv[F_NZ] = (float)nz;
        }
        fv[F_XI] = xI;
        fv[F_UX] = 0.5f * (float)ux; fv[F_UY] = 0.5f * (float)uy; fv[F_UZ] = 0.5f * (float)uz;
        fv[F_PH] = (float)(-2.0 * RP_PI * (ti - floor(ti)));
        fv[F_VX] = 0.5f * (float)vx; fv[F_VY] = 0.5f * (float)vy; fv[F_VZ] = 0.5f * (float)vz;
        fv[F_K] = (float)Kf;
    }
    // interleave with the partner facet j ^ 1 (FacetPair): the even lane
    // writes fields 0-7 of the pair, the odd lane fields 8-15; a missing odd
    // partner is the even facet with K = 0
    {
        const int lane1 = threadIdx.x & 1;
        const bool pok = __shfl_xor_sync(0xffffffffu, ok ? 1 : 0, 1) != 0;
        float pv[RP_NFIELD];
#pragma unroll
        for (int f = 0; f < RP_NFIELD; ++f) pv[f] = __shfl_xor_sync(0xffffffffu, fv[f], 1);
        const bool pair_ok = lane1 ? pok : ok;      // the pair's even facet exists
        if (pair_ok) {
            float e[RP_NFIELD], o[RP_NFIELD];        // even and odd facet of the pair
#pragma unroll
            for (int f = 0; f < RP_NFIELD; ++f) {
                e[f] = lane1 ? pv[f] : fv[f];
                const bool odd_ok = lane1 ? ok : pok;
                o[f] = odd_ok ? (lane1 ? fv[f] : pv[f]) : (f == F_K ? 0.f : e[f]);
            }
            FacetPair* pr = rec + ((size_t)s * rstride + j) / 2;
            const int h = lane1 * (RP_NFIELD / 4);  // first float4 this lane writes
#pragma unroll
            for (int i = 0; i < RP_NFIELD / 4; ++i) {
                const int f = 2 * (h + i);
                pr->v[h + i] = make_float4(e[f], o[f], e[f + 1], o[f + 1]);
            }
        }
        if constexpr (SPEC) {     // the pair's FacetSpec (even lane r, odd lane p)
            const float m[4] = {spR, spC, spI, spS};
            float pm[4], e[4], o[4];
#pragma unroll
            for (int f = 0; f < 4; ++f) pm[f] = __shfl_xor_sync(0xffffffffu, m[f], 1);
            const bool odd_ok = lane1 ? ok : pok;
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                e[f] = lane1 ? pm[f] : m[f];
                o[f] = odd_ok ? (lane1 ? m[f] : pm[f]) : e[f];
            }
            if (pair_ok) {
                FacetSpec* ps = spec + ((size_t)s * rstride + j) / 2;
                if (lane1) ps->p = make_float4(e[2], o[2], e[3], o[3]);
                else ps->r = make_float4(e[0], o[0], e[1], o[1]);
            }
        }
        if constexpr (T0) {       // the pair's FacetT0 (even lane); a missing odd facet adds zero
            const float pa = __shfl_xor_sync(0xffffffffu, t0a, 1), pdd = __shfl_xor_sync(0xffffffffu, t0d, 1);
            if (pair_ok && !lane1)
                t0rec[((size_t)s * rstride + j) / 2].v = make_float4(t0a, pok ? pa : 0.f, t0d, pok ? pdd : t0d);
        }
    }
    // the surface amplitude maximum of the trace (one atomic per chunk), the
    // chunk's radius and its range of xI, in one combined reduction
    float mx4[4] = {amax, ok ? rr : 0.f, ok ? -xI : -3e38f, ok ? xI : -3e38f};
    block_max_n<4>(mx4, shf);
    const float bmax = mx4[0];
    if (threadIdx.x == 0 && bmax > 0.f) atomic_max_pos(vmax + s, (double)bmax);
    const float R = mx4[1], xmn = -mx4[2], xmx = mx4[3];
    if (threadIdx.x == 0) {
        ChunkMeta m;
        m.cx = cx; m.cy = cy; m.cz = cz;
        m.R = R * (1.0f + 1e-6f) + 1e-4f;
        m.xmin = xmn; m.xmax = xmx;
        m.n = min(RP_CHUNK, n - k * RP_CHUNK);
        m.cfx = cfx; m.cfy = cfy; m.cfz = cfz;
        const double cc = (double)cfx * cfx + (double)cfy * cfy + (double)cfz * cfz;
        m.cch = (float)cc;
        m.ccl = (float)(cc - (double)m.cch);
        const double kb = dp.nidx / dp.dr;
        m.lo_off = (float)((double)xmn - kb * (double)m.R);
        m.hi_off = (float)((double)xmx + kb * (double)m.R);
        m.phase_ok = dp.nidx * dp.turn * (double)m.R < 40.0;    // |kt dT| <= kt R
        m.bbmin[0] = mnx; m.bbmin[1] = mny; m.bbmin[2] = mnz;
        m.bbmax[0] = mxx; m.bbmax[1] = mxy; m.bbmax[2] = mxz;
        meta[(size_t)s * mstride + k] = m;
    }
}

// Fixed-point accumulation of the surface leg (same scheme as the plain form).
// The surface of a trace concentrates in a few bins, so each block first sums
// its facets into a shared-memory window of RP_SFIX_WIN bins starting at the
// block's lowest bin (integer adds: order-free), then adds each non-zero bin
// to the trace with one global atomic; contributions beyond the window go to
// global memory directly.
#define RP_SFIX_WIN 128
#define RP_SFIX_PER 4
__global__ void __launch_bounds__(256) k_surf_fix32(int64_t nf, const int* __restrict__ nill,
                                                    const float* __restrict__ sx, const C32* __restrict__ sv,
                                                    const unsigned long long* __restrict__ vmax, int nr,
                                                    long long* __restrict__ acc, int single) {
    __shared__ unsigned long long hist[2 * RP_SFIX_WIN];
    __shared__ int sh_min[32];
    const int s = blockIdx.y;
    const int n = nill[s];
    const int64_t j0 = (int64_t)blockIdx.x * blockDim.x * RP_SFIX_PER;
    if (j0 >= n) return;                                  // uniform per block
    double vm = __longlong_as_double((long long)vmax[s]);
    if (!(vm > 0)) return;
    const double scale = ldexp(1.0, RP_FIX_BITS) / (2.0 * (double)n * vm);
    long long* a = acc + (size_t)s * nr * 2;
    int bl = INT_MAX;
    for (int k = 0; k < RP_SFIX_PER; ++k) {
        const int64_t j = j0 + (int64_t)k * blockDim.x + threadIdx.x;
        if (j < n) {
            double x = sx[(size_t)s * nf + j];
            if (x > -1.0 && x < (double)nr) bl = min(bl, (int)(long)x);
        }
    }
    for (int o = 16; o > 0; o >>= 1) bl = min(bl, __shfl_xor_sync(0xffffffffu, bl, o));
    if ((threadIdx.x & 31) == 0) sh_min[threadIdx.x >> 5] = bl;
    for (int i = threadIdx.x; i < 2 * RP_SFIX_WIN; i += blockDim.x) hist[i] = 0ull;
    __syncthreads();
    int blo = INT_MAX;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) blo = min(blo, sh_min[w]);
    for (int k = 0; k < RP_SFIX_PER; ++k) {
        const int64_t j = j0 + (int64_t)k * blockDim.x + threadIdx.x;
        if (j >= n) continue;
        double x = sx[(size_t)s * nf + j];
        if (!(x > -1.0) || x >= (double)nr) continue;
        long b = (long)x;
        // single (specular, genPhasorTrace): the whole phasor in the truncated bin
        double w = single ? 0.0 : x - (double)b;
        C32 v = sv[(size_t)s * nf + j];
        const long long q[4] = {llrint((double)v.x * (1.0 - w) * scale), llrint((double)v.y * (1.0 - w) * scale),
                                llrint((double)v.x * w * scale), llrint((double)v.y * w * scale)};
        for (int h = 0; h < 2 - single; ++h) {
            const long bb = b + h;
            if (h == 1 && bb >= nr) break;
            const long sl = bb - blo;
            if (sl >= 0 && sl < RP_SFIX_WIN) {
                atomicAdd(&hist[2 * sl], (unsigned long long)q[2 * h]);
                atomicAdd(&hist[2 * sl + 1], (unsigned long long)q[2 * h + 1]);
            } else {
                atomicAdd(reinterpret_cast<unsigned long long*>(a + 2 * bb), (unsigned long long)q[2 * h]);
                atomicAdd(reinterpret_cast<unsigned long long*>(a + 2 * bb + 1), (unsigned long long)q[2 * h + 1]);
            }
        }
    }
    __syncthreads();
    if (blo == INT_MAX) return;
    for (int i = threadIdx.x; i < 2 * RP_SFIX_WIN; i += blockDim.x) {
        const unsigned long long v = hist[i];
        const long bb = blo + (i >> 1);
        if (v != 0ull && bb < nr) atomicAdd(reinterpret_cast<unsigned long long*>(a + 2 * bb + (i & 1)), v);
    }
}

// Per-trace bounding box of illuminated facets and range of xI (fixed order).
struct TraceMeta {
    double bbmin[3], bbmax[3];
    float xmin, xmax;
    int nchunks, pad;
};

__global__ void k_tmeta32(const ChunkMeta* __restrict__ meta, int64_t mstride,
                          const int* __restrict__ nill, TraceMeta* __restrict__ tm) {
    __shared__ double shd[32];
    __shared__ float shf[32];
    const int s = blockIdx.x;
    const int nc = (nill[s] + RP_CHUNK - 1) / RP_CHUNK;
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    float xmn = 3e38f, xmx = -3e38f;
    for (int k = threadIdx.x; k < nc; k += blockDim.x) {
        const ChunkMeta& m = meta[(size_t)s * mstride + k];
        for (int a = 0; a < 3; ++a) { mn[a] = fmin(mn[a], m.bbmin[a]); mx[a] = fmax(mx[a], m.bbmax[a]); }
        xmn = fminf(xmn, m.xmin);
        xmx = fmaxf(xmx, m.xmax);
    }
    TraceMeta r;
    for (int a = 0; a < 3; ++a) {
        r.bbmin[a] = block_reduce(mn[a], MinOp(), shd);
        r.bbmax[a] = block_reduce(mx[a], MaxOp(), shd);
    }
    r.xmin = block_reduce(xmn, MinOpF(), shf);
    r.xmax = block_reduce(xmx, MaxOpF(), shf);
    r.nchunks = nc;
    if (threadIdx.x == 0) tm[s] = r;
}

// Per (trace, in-aperture target): FP32 normal, FP64 position and the bin
// window [bt0, bt0 + width) that bounds every pair of the trace (triangle
// inequality on the illuminated bounding box).
__global__ void k_tsetup32(const double* __restrict__ TG, int64_t nt, const int* __restrict__ tlist,
                           const int* __restrict__ ntl, int64_t tstride, const TraceMeta* __restrict__ tm,
                           const int* __restrict__ nill, DevParams dp, int* __restrict__ bt0,
                           int* __restrict__ maxw) {
    const int s = blockIdx.y;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ntl[s] || nill[s] == 0) return;
    const int64_t ti = tlist[(size_t)s * tstride + q];
    const double p[3] = {TG[ti], TG[nt + ti], TG[2 * nt + ti]};
    const TraceMeta m = tm[s];
    double dmin2 = 0, dmax2 = 0;
    for (int a = 0; a < 3; ++a) {
        double lo = m.bbmin[a] - p[a], hi = m.bbmax[a] - p[a];
        double c = (lo > 0) ? lo : ((hi < 0) ? -hi : 0.0);
        dmin2 += c * c;
        double f = fmax(fabs(lo), fabs(hi));
        dmax2 += f * f;
    }
    // bins per metre of Ttd: n (accumulateTarget) or c1/c2 (genRefrPhasor, ttype 0)
    const double kb = (TG[6 * nt + ti] == 0.0 ? dp.c1_over_c2 : dp.nidx) / dp.dr;
    double lo = (double)m.xmin + kb * sqrt(dmin2);
    double hi = (double)m.xmax + kb * sqrt(dmax2);
    int b0 = (int)floor(lo) - 2;
    int b1 = (int)floor(hi) + 3;
    b0 = max(b0, 0);
    b1 = min(b1, dp.nr);
    if (b1 < b0) b1 = b0;
    bt0[(size_t)s * tstride + q] = b0;
    atomicMax(maxw, b1 - b0);
}

// Per trace: the ttype-1 targets' count, the length of the leading run of
// the ordered target list below nt1 (the fast form's store holds ttype-1
// targets first).
__global__ void k_ntl1(const int* __restrict__ tlist, const int* __restrict__ ntl, int64_t tstride, int64_t nt1,
                       int nb, int* __restrict__ ntl1) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nb) return;
    const int* l = tlist + (size_t)s * tstride;
    int lo = 0, hi = ntl[s];            // first position with l[pos] >= nt1
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (l[mid] < nt1) lo = mid + 1; else hi = mid;
    }
    ntl1[s] = lo;
}

// ttype-0 targets: their phasor traces (rows [ntl1, ntl) of T, all facet-range
// parts) summed per bin in target order (FP64) into a dense trace per trace,
// in two passes.  Pass 1: the trace's targets in RP_T0_GROUPS consecutive
// groups (a fixed split of the trace's own list, so the sums never depend on
// the batch); a block adds its group's rows, one target after the other,
// into a dense FP64 partial (shared memory when it fits, else its slot of
// gpart).  Pass 2: the groups' partials summed in group order.
#define RP_T0_GROUPS 32
#define RP_T0_SMEM_MAX ((size_t)160 << 10)
__global__ void __launch_bounds__(256) k_t0_part32(const int* __restrict__ ntl1, const int* __restrict__ ntl,
                                                   int64_t tstride, const int* __restrict__ bt0,
                                                   const C32* __restrict__ T, int Wt, int nb, int nr,
                                                   double2* __restrict__ gpart, int use_smem) {
    extern __shared__ __align__(16) unsigned char t0sm[];
    const int g = blockIdx.x, s = blockIdx.y;
    double2* acc = use_smem ? reinterpret_cast<double2*>(t0sm) : gpart + ((size_t)s * RP_T0_GROUPS + g) * nr;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) acc[i] = make_double2(0.0, 0.0);
    __syncthreads();
    const int a = ntl1[s], n0 = ntl[s] - a;
    const int q0 = a + (int)((int64_t)n0 * g / RP_T0_GROUPS), q1 = a + (int)((int64_t)n0 * (g + 1) / RP_T0_GROUPS);
    for (int q = q0; q < q1; ++q) {
        const int b0 = bt0[(size_t)s * tstride + q];
        for (int o = threadIdx.x; o < Wt; o += blockDim.x) {
            const int i = b0 + o;
            if (i >= nr) break;
            double vr = 0.0, vi = 0.0;
            for (int p = 0; p < RP_PARTS; ++p) {
                const size_t ui = (((size_t)p * nb + s) * tstride + q) * Wt + o;
                const float4 u = reinterpret_cast<const float4*>(T)[ui];
                vr += (double)u.x + (double)u.z;
                vi += (double)u.y + (double)u.w;
            }
            double2 c = acc[i];
            c.x += vr;
            c.y += vi;
            acc[i] = c;
        }
        __syncthreads();    // the next target's row may cover the same bins
    }
    if (use_smem)
        for (int i = threadIdx.x; i < nr; i += blockDim.x) gpart[((size_t)s * RP_T0_GROUPS + g) * nr + i] = acc[i];
}

__global__ void k_t0_sum32(const double2* __restrict__ gpart, int nr, C32* __restrict__ sum0) {
    const int s = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nr) return;
    double vr = 0.0, vi = 0.0;
    for (int g = 0; g < RP_T0_GROUPS; ++g) {
        const double2 c = gpart[((size_t)s * RP_T0_GROUPS + g) * nr + i];
        vr += c.x;
        vi += c.y;
    }
    sum0[(size_t)s * nr + i] = C32{(float)vr, (float)vi};
}

// The ttype-0 targets' contribution: the summed trace convolved with the
// targets' chirp (genPhasorTrace + convolvePhasorChirpLinear per target,
// sim.cu:940-966, is linear and the same chirp for all, so one convolution
// of the sum per trace).  circ: specular mode with circular convolution,
// the nr-point convolution with genChirp's wrapped chirp CR (sim.cu:959).
__global__ void k_t0_conv32(const C32* __restrict__ sum0, int nr, const C32* __restrict__ C, PlanV<float> p2,
                            C32* __restrict__ r0, C32* __restrict__ scratch, size_t slot, int circ,
                            const C32* __restrict__ CR, PlanV<float> pR) {
    const int s = blockIdx.x;
    C32* base = scratch + (size_t)s * slot;
    const int M = 1 << p2.log2M;
    C32* x = base;
    C32* wa = x + M;
    C32* wb = wa + M;
    C32* in = wb + M;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) in[i] = sum0[(size_t)s * nr + i];
    __syncthreads();
    if (circ) conv_circular_block<float>(in, CR, pR, nr, x, wa, wb, r0 + (size_t)s * nr);
    else conv_linear_block<float>(in, C, p2, nr, x, wa, wb, r0 + (size_t)s * nr, 1.0f);
}

// Single-batch pair kernel: the batch's constants live in the parameter
// bank.  Persistent: blocks take (trace, target block, part) items from a
// work counter until all are done.  SUB: the wave's parts are split further
// (2^lparts parts, pair_sub), an instance of its own so that the common
// kernel keeps its compile-time part count.
template <int NT, int ILP, int MINB, bool ORTHO, bool SUB = false>
__global__ void __launch_bounds__(RP_PAIR_THREADS, MINB)
k_pairs32(const __grid_constant__ PairArgs A) {
    RP_PAIR_SMEM_DECL
    const int lp = SUB ? A.lparts : RP_LPARTS;
    const unsigned int items = ((unsigned)A.nb * A.tblocks) << lp;
    for (;;) {
        if (tid == 0) s_item = atomicAdd(A.work, 1u);
        __syncthreads();
        const unsigned int item = s_item;
        __syncthreads();
        if (item >= items) break;
        if constexpr (SUB) {
            const int part = item & ((1u << lp) - 1u);
            const int tb = (item >> lp) % A.tblocks;
            const int s = (item >> lp) / A.tblocks;
            if (!pair_item<NT, ILP, ORTHO, false, RP_WIN_WIDE>(A, s, tb, part, bars, phase, lp)) break;
        } else {
            const int part = item % RP_PARTS;
            const int tb = (item / RP_PARTS) % A.tblocks;
            const int s = item / (RP_PARTS * A.tblocks);
            if (!pair_item<NT, ILP, ORTHO, false, RP_WIN_WIDE>(A, s, tb, part, bars, phase)) break;
        }
    }
    RP_PAIR_SMEM_END
}

// Folds a wave's facet sub-parts back into its RP_PARTS parts: part p's row
// element becomes the compensated sum of sub-parts p sub ... p sub + sub - 1
// (in that order) at part p's place, so the compression reads RP_PARTS
// parts as always.  A thread owns one element of every part and reads all
// its sub-parts before it writes, so the fold runs in place.
__global__ void k_fold_parts(float4* __restrict__ T, int64_t slot, int sub) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < slot;
         e += (int64_t)gridDim.x * blockDim.x) {
        float4 out[RP_PARTS];
#pragma unroll
        for (int p = 0; p < RP_PARTS; ++p) {
            float4 acc = T[(int64_t)p * sub * slot + e];
            for (int j = 1; j < sub; ++j) {
                const float4 u = T[((int64_t)p * sub + j) * slot + e];
                acc = comp_add(acc, u.x, u.y);
                acc.z = __fadd_rn(acc.z, u.z);
                acc.w = __fadd_rn(acc.w, u.w);
            }
            out[p] = acc;
        }
#pragma unroll
        for (int p = 0; p < RP_PARTS; ++p) T[(int64_t)p * slot + e] = out[p];
    }
}

// ---------------------------------------------------------- compression --
// Per (trace, target): T = sum of the facet-range parts (fixed order) placed
// at its window; Ptarg = linconv(T, chirp2); contribution =
// convolveComplex(-T/sqrt(P), Ptarg) -> Z row (complex64, dense nr).  In
// specular mode (T2 != null) Psour is -T2/sqrt(P), the outbound leg's trace.
__global__ void k_conv32(const int* __restrict__ ntl, int64_t tstride, int nb, const int* __restrict__ bt0,
                         const C32* __restrict__ T, const C32* __restrict__ T2, int Wt, C32* __restrict__ Z,
                         const C32* __restrict__ C2, PlanV<float> p2, PlanV<float> pN, int crop_K, int crop_all,
                         int nr, float sig_scale, C32* __restrict__ scratch, size_t slot) {
    C32* base = scratch + (size_t)blockIdx.x * slot;
    const int M = max(1 << p2.log2M, 1 << pN.log2M);
    C32* x = base;
    C32* wa = x + M;
    C32* wb = wa + M;
    C32* A = wb + M;
    C32* B = A + M;
    C32* tr = B + M;        // dense nr
    C32* ptarg = tr + nr;   // nr
    C32* tr2 = ptarg + nr;  // nr (specular)
    const int64_t items = (int64_t)nb * tstride;
    for (int64_t it = blockIdx.x; it < items; it += gridDim.x) {
        const int s = (int)(it / tstride);
        const int q = (int)(it % tstride);
        if (q >= ntl[s]) continue;
        const int b0 = bt0[(size_t)s * tstride + q];
        for (int i = threadIdx.x; i < nr; i += blockDim.x) {
            C32 v{0.f, 0.f};
            const int o = i - b0;
            if (o >= 0 && o < Wt) {
                for (int p = 0; p < RP_PARTS; ++p) {
                    const size_t ui = (((size_t)p * nb + s) * tstride + q) * Wt + o;
                    const float4 u = reinterpret_cast<const float4*>(T)[ui];
                    v.x += u.x + u.z;
                    v.y += u.y + u.w;
                }
            }
            tr[i] = v;
            if (T2) {
                C32 u2{0.f, 0.f};
                if (o >= 0 && o < Wt)
                    for (int p = 0; p < RP_PARTS; ++p) {
                        const size_t ui = (((size_t)p * nb + s) * tstride + q) * Wt + o;
                        const float4 u = reinterpret_cast<const float4*>(T2)[ui];
                        u2.x += u.x + u.z;
                        u2.y += u.y + u.w;
                    }
                tr2[i] = u2;
            }
        }
        __syncthreads();
        conv_linear_block<float>(tr, C2, p2, nr, x, wa, wb, ptarg, 1.0f);
        conv_complex_block<float>(T2 ? tr2 : tr, ptarg, pN, nr, crop_K, crop_all, A, B, wa, wb,
                                  Z + ((size_t)s * tstride + q) * nr, sig_scale);
    }
}

// The targets' u summed over the splits of each trace (split order, FP64),
// written over split 0 (each thread owns its element).  Wide, so the FP64
// sums spread over every SM.
__global__ void k_usum32(const int* __restrict__ nill, const int* __restrict__ ntl, C32* __restrict__ part,
                         int nsplit, int n2) {
    const int s = blockIdx.y;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n2) return;
    const int ns = nill[s] > 0 ? (ntl[s] + RP_CONV_SPLIT - 1) / RP_CONV_SPLIT : 0;
    C32* z = part + (size_t)s * nsplit * n2 + k;
    double vr = 0.0, vi = 0.0;
    if (k < n2 - 1)
        for (int q = 0; q < ns; ++q) {
            const C32 u = z[(size_t)q * n2];
            vr += u.x;
            vi += u.y;
        }
    z[0] = C32{(float)vr, (float)vi};
}

// Per trace (one block): the summed u (split 0 after k_usum32), then cropSpectrum and the inverse N-point DFT as the circular
// convolution with the crop kernel h (its M-point spectrum Hs, M = 4nr >=
// 2N - 1: linear convolution, then circ[n] = lin[n] + lin[n + N]),
// takeEveryOtherComplex (circ[2j]) and sig = refl + that (FP64).  W: M
// complex values in shared memory, or (gW != null) in this trace's slot of
// global scratch.
__global__ void __launch_bounds__(512, 1)
k_trace_m32(const int* __restrict__ nill, const int* __restrict__ ntl, const C32* __restrict__ refl,
            const C32* __restrict__ part, int nsplit, int nr, const Cplx<float>* __restrict__ Hs,
            Cplx<float>* __restrict__ gW, void* __restrict__ out, int out64, int s0,
            const C32* __restrict__ r0) {
    extern __shared__ __align__(16) unsigned char tsm[];
    const int s = blockIdx.x;
    const int n2 = 2 * nr, N = n2 - 1, M = 2 * n2;
    Cplx<float>* W = gW ? gW + (size_t)s * M : reinterpret_cast<Cplx<float>*>(tsm);
    const bool any = nill[s] > 0;
    const C32* z = part + (size_t)s * nsplit * n2;
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        const C32 u = k < N ? z[k] : C32{0.f, 0.f};
        W[swz(k)] = Cplx<float>{u.x, u.y};
    }
    __syncthreads();
    block_dif_s<float>(W, M);
    for (int k = threadIdx.x; k < M; k += blockDim.x) W[swz(k)] = c_mul(W[swz(k)], Hs[k]);
    __syncthreads();
    block_dit_s<float>(W, M);
    for (int j = threadIdx.x; j < nr; j += blockDim.x) {
        double vr = 0.0, vi = 0.0;
        if (any) {
            const C32 r = refl[(size_t)s * nr + j];
            const Cplx<float> a = W[swz(2 * j)], b = W[swz(2 * j + N)];
            vr = (double)r.x + ((double)a.x + (double)b.x);
            vi = (double)r.y + ((double)a.y + (double)b.y);
            if (r0) {       // ttype-0 targets
                vr += (double)r0[(size_t)s * nr + j].x;
                vi += (double)r0[(size_t)s * nr + j].y;
            }
        }
        const size_t o = (size_t)(s0 + s) * nr + j;
        if (out64) reinterpret_cast<C64*>(out)[o] = C64{vr, vi};
        else reinterpret_cast<float2*>(out)[o] = make_float2((float)vr, (float)vi);
    }
}

__global__ void k_surf_conv32(const long long* __restrict__ acc, const int* __restrict__ nill,
                              const unsigned long long* __restrict__ vmax, int disable, int nr,
                              const C32* __restrict__ C1, PlanV<float> p2, C32* __restrict__ refl,
                              C32* __restrict__ scratch, size_t slot) {
    const int s = blockIdx.x;
    C32* base = scratch + (size_t)s * slot;
    const int M = 1 << p2.log2M;
    C32* x = base;
    C32* wa = x + M;
    C32* wb = wa + M;
    C32* in = wb + M;
    const int n = nill[s];
    double vm = __longlong_as_double((long long)vmax[s]);
    double inv = (n > 0 && vm > 0) ? (2.0 * (double)n * vm) / ldexp(1.0, RP_FIX_BITS) : 0.0;
    const long long* a = acc + (size_t)s * nr * 2;
    for (int i = threadIdx.x; i < nr; i += blockDim.x)
        in[i] = disable ? C32{0.f, 0.f} : C32{(float)((double)a[2 * i] * inv), (float)((double)a[2 * i + 1] * inv)};
    __syncthreads();
    conv_linear_block<float>(in, C1, p2, nr, x, wa, wb, refl + (size_t)s * nr, 1.0f);
}

// sig = refl + sum_q Z_q (target order), accumulated in FP64.
__global__ void k_sum32(const int* __restrict__ nill, const int* __restrict__ ntl, int64_t tstride,
                        const C32* __restrict__ refl, const C32* __restrict__ Z, int nr,
                        void* __restrict__ out, int out64, int s0, const C32* __restrict__ r0) {
    const int s = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nr) return;
    double vr = 0.0, vi = 0.0;
    if (nill[s] > 0) {
        C32 r = refl[(size_t)s * nr + i];
        vr = r.x; vi = r.y;
        if (r0) {           // ttype-0 targets
            vr += r0[(size_t)s * nr + i].x;
            vi += r0[(size_t)s * nr + i].y;
        }
        const int n = ntl[s];
        const C32* z = Z + (size_t)s * tstride * nr + i;
        for (int q = 0; q < n; ++q) {
            C32 u = z[(size_t)q * nr];
            vr += u.x;
            vi += u.y;
        }
    }
    const size_t o = (size_t)(s0 + s) * nr + i;
    if (out64) reinterpret_cast<C64*>(out)[o] = C64{vr, vi};
    else reinterpret_cast<float2*>(out)[o] = make_float2((float)vr, (float)vi);
}

// ------------------------------------------------------------- driver ----
struct FastLayout {
    int nb;
    int64_t tstride;
    int64_t fstride;     // illuminated facets a trace can hold (host bound, <= nf)
    int64_t rstride;     // records per trace (fstride rounded to chunks)
    int64_t mstride;     // chunks per trace
    int Wt;
    int slots;
    size_t slot, surf_slot;
};

template <class Aa>
void fast_take_setup(Aa& a, const rp_scene* sc, const FastLayout& L) {
    const int64_t nf = std::max<int64_t>(sc->nf, 1), nt = std::max<int64_t>(sc->nt, 1);
    const int nr = sc->nr;
    const int tiles = (int)((std::max(nf, nt) + RP_TILE - 1) / RP_TILE);
    a.template take<uint8_t>((size_t)L.nb * nf);
    a.template take<int>((size_t)L.nb * tiles);
    a.template take<int>(L.nb);                             // nill
    a.template take<int>(L.nb);                             // ntl
    a.template take<unsigned long long>(L.nb);              // vmax
    a.template take<int>((size_t)L.nb * L.fstride);         // idx
    a.template take<FacetPair>((size_t)L.nb * L.rstride / 2);    // records (facet pairs)
    if (sc->dp.specular) a.template take<FacetSpec>((size_t)L.nb * L.rstride / 2);
    if (sc->nt1 < sc->nt) {
        a.template take<FacetT0>((size_t)L.nb * L.rstride / 2);
        a.template take<int>(L.nb);                         // ntl1
    }
    a.template take<ChunkMeta>((size_t)L.nb * L.mstride);   // chunk meta
    a.template take<double>((size_t)L.nb * 4);              // trace origins
    a.template take<float>((size_t)L.nb * L.fstride);       // surface x
    a.template take<C32>((size_t)L.nb * L.fstride);         // surface v
    a.template take<TraceMeta>(L.nb);
    a.template take<uint8_t>((size_t)L.nb * nt);            // target flags
    a.template take<int>((size_t)L.nb * nt);                // tlist
    a.template take<int>((size_t)L.nb * L.tstride);         // bt0
    a.template take<int>(8);                                // maxw, work, err[2], conv work
    a.template take<long long>((size_t)L.nb * nr * 2);      // surface fixed point
    a.template take<C32>((size_t)L.nb * nr);                // refl
    a.template take<C32>((size_t)L.nb * L.surf_slot);       // surface conv scratch
}

// Storage mode of the range compression (k_conv32s): 0 X and W in shared
// memory (2 x 2nr complex64 = 32 nr bytes, 128 KiB at nr = 4096), 1 the
// transforms in shared memory and X parked in global scratch (nr = 8192),
// 2 both in global scratch (nr >= 16384), 3 the Bluestein kernel k_conv32
// (nr not a power of two).
int conv_mode(const rp_scene* sc) {
    if (!sc->smem_conv) return 3;
    if (sc->nr <= 4096) return 0;
    if (sc->nr <= 8192) return 1;
    return 2;
}

// Complex values in one block's slot of the global compression scratch: X
// (2nr) in mode 1, X and W (2nr each) in mode 2.
size_t conv_gslot(const rp_scene* sc) {
    const int m = conv_mode(sc);
    return m == 1 ? (size_t)2 * sc->nr : (m == 2 ? (size_t)4 * sc->nr : 0);
}

// The per-trace crop stage (k_trace_m32) keeps its M = 4nr values in shared
// memory up to this size, else in a per-trace slot of global scratch.
const size_t kTraceSmemMax = (size_t)200 << 10;
bool trace_m_global(const rp_scene* sc) { return (size_t)4 * sc->nr * sizeof(C32) > kTraceSmemMax; }

int64_t conv_splits(int64_t tstride) { return (tstride + RP_CONV_SPLIT - 1) / RP_CONV_SPLIT; }

template <class Aa>
void fast_take_pairs(Aa& a, const rp_scene* sc, const FastLayout& L) {
    a.template take<C32>((size_t)2 * RP_PARTS * L.nb * L.tstride * L.Wt);   // T parts (high, low)
    if (sc->dp.specular) a.template take<C32>((size_t)2 * RP_PARTS * L.nb * L.tstride * L.Wt);   // T2 parts
    if (sc->dp.cmode == 2)        // direct sums: the facet groups' partial traces
        a.template take<double2>((size_t)L.nb * RP_DS_GROUPS * sc->nr);
    if (sc->nt1 < sc->nt) {       // ttype-0 sum, r0, scratch, group partials
        a.template take<C32>((size_t)L.nb * (2 * sc->nr + L.surf_slot));
        a.template take<double2>((size_t)L.nb * RP_T0_GROUPS * sc->nr);
    }
    if (conv_mode(sc) <= 2) {
        a.template take<C32>((size_t)L.nb * conv_splits(L.tstride) * 2 * sc->nr);   // per-split sums of u
        if (trace_m_global(sc)) a.template take<C32>((size_t)L.nb * 4 * sc->nr);   // per-trace crop stage
        // global compression scratch: one slot per SM (a wave takes one region
        // for all its segments, sized here per segment as an upper bound)
        if (conv_mode(sc) >= 1) a.template take<C32>((size_t)sc->sm_count * conv_gslot(sc));
    } else {
        a.template take<C32>((size_t)L.nb * L.tstride * sc->nr);        // Z
        a.template take<C32>((size_t)L.slots * L.slot);                  // conv scratch
    }
}

FastLayout fast_layout(const rp_scene* sc, int nb, int64_t tstride, int Wt, int64_t fstride) {
    FastLayout L;
    L.nb = nb;
    L.tstride = std::max<int64_t>(tstride, 1);
    L.fstride = std::max<int64_t>(std::min<int64_t>(fstride, sc->nf), 1);
    L.mstride = std::max<int64_t>((L.fstride + RP_CHUNK - 1) / RP_CHUNK, 1);
    L.rstride = L.mstride * RP_CHUNK;
    L.Wt = std::max(Wt, 1);
    const int M = std::max(sc->plan2.M(), sc->planN.M());
    L.slot = (size_t)5 * M + 3 * sc->nr;
    L.surf_slot = (size_t)3 * sc->plan2.M() + sc->nr;
    L.slots = std::max(1, 2 * sc->sm_count);
    return L;
}

// Scratch of one wave (the segments whose pair stage shares one launch):
// the 64-scene uneven batch at 8 traces per scene fits one wave.
const size_t kFastBudget = (size_t)64 << 30;


// Pair-kernel instantiation: sinc degree x frame kind x (ILP facet pairs per
// step, resident blocks per SM).  cfg 0: 2 x 3, 1: 2 x 2, 2: 3 x 2, 3: 4 x 2.
template <int NT>
void (*pick_cfg(int cfg, bool ortho))(const PairArgs) {
    if (ortho) {
        switch (cfg) {
            case 1: return k_pairs32<NT, 2, 2, true>;
            case 2: return k_pairs32<NT, 3, 2, true>;
            case 3: return k_pairs32<NT, 4, 2, true>;
            default: return k_pairs32<NT, 2, 3, true>;
        }
    }
    switch (cfg) {
        case 1: return k_pairs32<NT, 2, 2, false>;
        case 2: return k_pairs32<NT, 3, 2, false>;
        case 3: return k_pairs32<NT, 4, 2, false>;
        default: return k_pairs32<NT, 2, 3, false>;
    }
}

void (*pick_pair_kernel(int deg, int cfg, bool ortho, bool sub = false))(const PairArgs) {
    if (sub) {      // split parts: the default shape (4 facet pairs per step, 2 blocks per SM)
        switch (deg) {
            case 3: return ortho ? k_pairs32<3, 4, 2, true, true> : k_pairs32<3, 4, 2, false, true>;
            case 4: return ortho ? k_pairs32<4, 4, 2, true, true> : k_pairs32<4, 4, 2, false, true>;
            case 5: return ortho ? k_pairs32<5, 4, 2, true, true> : k_pairs32<5, 4, 2, false, true>;
            case 6: return ortho ? k_pairs32<6, 4, 2, true, true> : k_pairs32<6, 4, 2, false, true>;
            default: return ortho ? k_pairs32<0, 4, 2, true, true> : k_pairs32<0, 4, 2, false, true>;
        }
    }
    switch (deg) {
        case 3: return pick_cfg<3>(cfg, ortho);
        case 4: return pick_cfg<4>(cfg, ortho);
        case 5: return pick_cfg<5>(cfg, ortho);
        case 6: return pick_cfg<6>(cfg, ortho);
        default: return pick_cfg<0>(cfg, ortho);
    }
}

// Degree of the polynomial in t = a^2 that approximates sin(a)/a to 1e-6
// (maximum absolute error of the Chebyshev projection below) for |a| <=
// amax (0: use the special-function unit).  A directivity is a product of
// four such factors, so amplitudes carry at most ~4e-6 relative error.
// Measured maxima: degree 3 at 1.6: 8.8e-7; 4 at 2.5: 4.2e-7; 5 at 4.0:
// 1.0e-6; 6 at 5.0: 4.0e-7.  variant 1 forces the special-function path.
int sinc_degree(double amax, int variant) {
    if (variant == 1) return 0;
    if (amax <= 1.6) return 3;
    if (amax <= 2.5) return 4;
    if (amax <= 4.0) return 5;
    if (amax <= 5.0) return 6;
    return 0;
}

// Chebyshev projection of s(t) = sin(sqrt t)/sqrt t on [0, T] (64 nodes,
// degree D), converted to monomial coefficients in t: near-minimax, own
// construction from the Chebyshev expansion of a smooth function.
void sinc_poly(double T, int D, double* mono) {
    const int N = 64;
    double c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < N; ++k) {
        const double th = RP_PI * (k + 0.5) / N;
        const double u = std::cos(th);
        const double t = 0.5 * T * (u + 1.0);
        const double a = std::sqrt(t);
        const double f = (a > 1e-12) ? std::sin(a) / a : 1.0;
        for (int j = 0; j <= D; ++j) c[j] += f * std::cos(j * th);
    }
    for (int j = 0; j <= D; ++j) c[j] *= 2.0 / N;
    c[0] *= 0.5;
    // sum_j c_j T_j(u) -> monomials in u (T_{j+1} = 2u T_j - T_{j-1})
    double Tm[8][8] = {};
    Tm[0][0] = 1.0;
    if (D >= 1) Tm[1][1] = 1.0;
    for (int j = 2; j <= D; ++j)
        for (int i = 0; i <= j; ++i) Tm[j][i] = (i ? 2.0 * Tm[j - 1][i - 1] : 0.0) - Tm[j - 2][i];
    double pu[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int j = 0; j <= D; ++j)
        for (int i = 0; i <= j; ++i) pu[i] += c[j] * Tm[j][i];
    // u = 2t/T - 1 = alpha t + beta -> monomials in t (binomial expansion)
    const double al = 2.0 / T, be = -1.0;
    for (int i = 0; i < 8; ++i) mono[i] = 0.0;
    for (int i = 0; i <= D; ++i) {
        double binom = 1.0;
        for (int k = 0; k <= i; ++k) {
            // C(i,k) al^k be^(i-k)
            mono[k] += pu[i] * binom * std::pow(al, k) * std::pow(be, i - k);
            binom = binom * (i - k) / (k + 1);
        }
    }
}

// ---------------------------------------------------------- autotuner ----
// (multi, degree) -> configuration, for the process.  Probing launches the
// candidate kernels on the real inputs (results are discarded and the
// outputs re-zeroed), so only timing depends on the choice.
std::mutex g_tune_mu;
std::map<std::pair<int, int>, int> g_tuned;
int g_autotune = -1;    // -1: not decided yet (env), 0 off, 1 on

bool autotune_on() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    if (g_autotune < 0) g_autotune = getenv("RP_PAIR_CFG") ? 0 : 1;
    return g_autotune == 1;
}

int tuned_lookup(int multi, int deg) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find({multi, deg});
    return it == g_tuned.end() ? -1 : it->second;
}

void tuned_store(int multi, int deg, int cfg) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[{multi, deg}] = cfg;
}

// ------------------------------------------------------------- segments ----
// A segment is up to 64 traces of one scene processed as one batch; a wave
// is a set of segments (possibly of different scenes) whose scratch fits the
// budget and whose pair stage runs as one launch.
struct Seg {
    rp_scene* sc = nullptr;
    const double* trb = nullptr;   // device trace rows of this segment
    int64_t s0 = 0;                // first row in the job's output
    int nb = 0;
    int64_t tmax = 0;
    int64_t fmax = 0;              // illuminated-facet capacity per trace (host bound)
    int wmax = 0;                  // target-window width, host bound over the segment's traces
    void* d_out = nullptr;
    int out64 = 0;
    int64_t* h_counts = nullptr;
    int deg = 0;
    const double* coef = nullptr;
    const double* coefr = nullptr;
    FastLayout Lw, L;
    // setup stage
    uint8_t* fflags; int* tcnt; int* nill; int* ntl; unsigned long long* vmax;
    double* org; int* idx; FacetPair* rec; ChunkMeta* meta; float* sxv; C32* sv; TraceMeta* tm; uint8_t* tflags;
    FacetSpec* spec = nullptr;     // specular mode
    FacetT0* t0rec = nullptr;      // ttype-0 targets present
    int* ntl1 = nullptr;           // ttype-1 targets per trace (= ntl without ttype-0 targets)
    int* tlist; int* bt0; int* misc; long long* acc; C32* refl; C32* sscr;
    // pair stage
    int Wt = 1;
    int nsplit = 0;
    int cmode = 0;          // compression storage mode (conv_mode)
    bool pairs = false;
    C32* T = nullptr; C32* Z = nullptr; C32* cscr = nullptr; C32* part = nullptr;
    int sub = 1;            // facet sub-splits per part (pair_sub)
    int64_t cbase = 0;      // first trace of the segment's job over all jobs of the call
    // row elements of T (and T2); each is {high, low}, two C32
    int64_t row_elems() const { return (int64_t)RP_PARTS * sub * nb * L.tstride * Wt; }
    C32* T2 = nullptr;      // specular mode: outbound-leg parts
    C32* sum0 = nullptr; C32* r0 = nullptr; C32* t0scr = nullptr;   // ttype-0 targets
    double2* t0part = nullptr;
    double2* dpart = nullptr;       // specular mode without convolution: direct-sum partials
    C32* tscr = nullptr;    // per-trace crop-stage scratch (nr > 4096)
};

struct SceneConst {
    int deg = 0;
    double coef[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    double coefr[8] = {0, 0, 0, 0, 0, 0, 0, 0};   // specular: facetReradiation's sinc on [0, pi fs / lam]
};

SceneConst scene_const(const rp_scene* sc) {
    SceneConst k;
    const double pik_d = RP_PI * (RP_PI_F * sc->dp.fs / sc->dp.lam);
    k.deg = sinc_degree(pik_d, sc->pair_variant);
    if (k.deg > 0) sinc_poly(pik_d * pik_d, k.deg, k.coef);
    // the reradiation argument is at most pi fs / lam < pik: the same degree
    // fits it at least as well
    const double pikr = RP_PI * sc->dp.fs / sc->dp.lam;
    if (k.deg > 0) sinc_poly(pikr * pikr, k.deg, k.coefr);
    return k;
}

size_t seg_setup_bytes(const rp_scene* sc, const FastLayout& L) {
    ArenaPlan a;
    fast_take_setup(a, sc, L);
    return a.off + 256;
}

size_t seg_pair_bytes(const rp_scene* sc, const FastLayout& L) {
    ArenaPlan a;
    fast_take_pairs(a, sc, L);
    return a.off + 256;
}

// Setup stage of one segment: cull and compact facets, facet records and
// chunk metadata, surface bins, target list, target windows (maxw in misc[0]).
void seg_setup(Seg& g, Arena& a, cudaStream_t st) {
    rp_scene* sc = g.sc;
    const int64_t nf = sc->nf, nt = sc->nt;
    const int nr = sc->nr, nb = g.nb;
    const DevParams& dp = sc->dp;
    const FastLayout& Lw = g.Lw;
    const int64_t nfa = std::max<int64_t>(nf, 1), nta = std::max<int64_t>(nt, 1);
    const int tiles = (int)((std::max(nfa, nta) + RP_TILE - 1) / RP_TILE);
    g.fflags = a.take<uint8_t>((size_t)nb * nfa);
    g.tcnt = a.take<int>((size_t)nb * tiles);
    g.nill = a.take<int>(nb);
    g.ntl = a.take<int>(nb);
    g.vmax = a.take<unsigned long long>(nb);
    g.idx = a.take<int>((size_t)nb * Lw.fstride);
    g.rec = a.take<FacetPair>((size_t)nb * Lw.rstride / 2);
    g.spec = dp.specular ? a.take<FacetSpec>((size_t)nb * Lw.rstride / 2) : nullptr;
    const bool t0 = sc->nt1 < nt;
    g.t0rec = t0 ? a.take<FacetT0>((size_t)nb * Lw.rstride / 2) : nullptr;
    g.meta = a.take<ChunkMeta>((size_t)nb * Lw.mstride);
    g.org = a.take<double>((size_t)nb * 4);
    g.sxv = a.take<float>((size_t)nb * Lw.fstride);
    g.sv = a.take<C32>((size_t)nb * Lw.fstride);
    g.tm = a.take<TraceMeta>(nb);
    g.tflags = a.take<uint8_t>((size_t)nb * nta);
    g.ntl1 = t0 ? a.take<int>(nb) : g.ntl;
    g.tlist = a.take<int>((size_t)nb * nta);
    g.bt0 = a.take<int>((size_t)nb * Lw.tstride);
    g.misc = a.take<int>(8);
    g.acc = a.take<long long>((size_t)nb * nr * 2);
    g.refl = a.take<C32>((size_t)nb * nr);
    g.sscr = a.take<C32>((size_t)nb * Lw.surf_slot);
    const double* trb = g.trb;
    cudaMemsetAsync(g.vmax, 0, sizeof(unsigned long long) * nb, st);
    cudaMemsetAsync(g.misc, 0, sizeof(int) * 8, st);
    cudaMemsetAsync(g.acc, 0, sizeof(long long) * nb * nr * 2, st);
    if (nf > 0) {
        k_cull_count<<<dim3((unsigned)((nf + RP_TILE - 1) / RP_TILE), nb), RP_TILE_THREADS, 0, st>>>(
            sc->d_sorted, nf, trb, dp.ap_rad, g.fflags, g.tcnt, reinterpret_cast<const double4*>(sc->d_tiles_sorted));
        RP_LAUNCHED();
        compact_flags(g.fflags, nf, nb, g.tcnt, g.nill, g.idx, Lw.fstride, true, st, g.misc + 6);
        auto kf = dp.specular ? (t0 ? k_facets32<true, true> : k_facets32<true, false>)
                              : (t0 ? k_facets32<false, true> : k_facets32<false, false>);
        kf<<<dim3((unsigned)Lw.mstride, nb), RP_CHUNK, 0, st>>>(
            sc->d_sorted, nfa, Lw.fstride, g.idx, g.nill, trb, dp, g.rec, g.meta, Lw.rstride, Lw.mstride, g.sxv, g.sv,
            g.vmax,
            g.org, sc->d_order, g.spec, g.t0rec);
        RP_LAUNCHED();
        k_surf_fix32<<<dim3((unsigned)((Lw.fstride + 256 * RP_SFIX_PER - 1) / (256 * RP_SFIX_PER)), nb), 256, 0,
                       st>>>(Lw.fstride, g.nill, g.sxv, g.sv, g.vmax, nr, g.acc, dp.specular);
        RP_LAUNCHED();
        k_tmeta32<<<nb, 256, 0, st>>>(g.meta, Lw.mstride, g.nill, g.tm);
        RP_LAUNCHED();
    } else {
        cudaMemsetAsync(g.nill, 0, sizeof(int) * nb, st);
    }
    if (nt > 0) {
        k_target_flags<<<dim3((unsigned)((nt + 255) / 256), nb), 256, 0, st>>>(sc->d_targets_fast, nt, trb,
                                                                            dp.ap_rad, g.tflags);
        RP_LAUNCHED();
        compact_flags(g.tflags, nt, nb, g.tcnt, g.ntl, g.tlist, Lw.tstride, false, st, g.misc + 6);
        if (t0) {
            k_ntl1<<<(nb + 63) / 64, 64, 0, st>>>(g.tlist, g.ntl, Lw.tstride, sc->nt1, nb, g.ntl1);
            RP_LAUNCHED();
        }
        if (nf > 0) {
            k_tsetup32<<<dim3((unsigned)((Lw.tstride + 255) / 256), nb), 256, 0, st>>>(
                sc->d_targets_fast, nt, g.tlist, g.ntl, Lw.tstride, g.tm, g.nill, dp, g.bt0, g.misc);
            RP_LAUNCHED();
        }
    } else {
        cudaMemsetAsync(g.ntl, 0, sizeof(int) * nb, st);
        if (g.ntl1 != g.ntl) cudaMemsetAsync(g.ntl1, 0, sizeof(int) * nb, st);
    }
}

PairArgs seg_pair_args(const Seg& g) {
    const rp_scene* sc = g.sc;
    const DevParams& dp = sc->dp;
    const int nr = sc->nr;
    PairArgs P;
    P.rec = g.rec; P.meta = g.meta; P.org = g.org; P.rstride = g.Lw.rstride; P.mstride = g.Lw.mstride;
    P.nill = g.nill; P.ntl = g.ntl1; P.tlist = g.tlist; P.tstride = g.L.tstride;
    P.TG = sc->d_targets_fast; P.nt = sc->nt; P.PR = sc->d_prisms; P.np = sc->np;
    P.bt0 = g.bt0; P.T = g.T; P.Wt = g.Wt; P.nb = g.nb;
    P.tblocks = (int)((g.L.tstride + RP_PAIR_THREADS - 1) / RP_PAIR_THREADS);
    P.lparts = RP_LPARTS;
    for (int k = g.sub; k > 1; k >>= 1) ++P.lparts;
    P.work = reinterpret_cast<unsigned int*>(g.misc + 1);
    P.err = reinterpret_cast<unsigned int*>(g.misc + 2);
    P.spin_limit = sc->spin_limit;
    P.stall_copies = sc->stall_copies;
    P.nr_f = (float)nr; P.nr = nr; P.nr1 = nr - 1;
    P.kb = (float)(dp.nidx / dp.dr);
    P.kt = (float)(dp.nidx * dp.turn);
    P.kr = (float)(-2.0 * RP_PI * dp.nidx * dp.turn);
    const double pik_d = RP_PI * (RP_PI_F * dp.fs / dp.lam);
    P.pik = (float)pik_d;
    P.pik2 = (float)(pik_d * pik_d);
    // the kernel's polynomial argument is t' = a^2 / pik^2 in [0, 1]
    for (int k = 0; k < 8; ++k) P.sc[k] = (float)(g.coef[k] * std::pow(pik_d * pik_d, k));
    P.ealpha = dp.lossless ? 0.f : (float)(-2.0 * dp.alpha2 * 1.4426950408889634);
    P.eks = dp.lossless ? 0.f : (float)(-2.0 * dp.ks * dp.ks * 1.4426950408889634);
    const double ktd = dp.nidx * dp.turn, kbd = dp.nidx / dp.dr;
    P.kth = (float)ktd; P.ktl = (float)(ktd - (double)P.kth);
    P.kbh = (float)kbd; P.kbl = (float)(kbd - (double)P.kbh);
    P.lossless = dp.lossless;
    // specular mode; lossless skips the reradiation factors with the rest of
    // compRefrEnergyIn/Out (a polynomial of 1, or a zero argument)
    P.spec = g.spec; P.T2 = g.T2;
    const double pikr = RP_PI * dp.fs / dp.lam;
    const bool rr = dp.specular && !dp.lossless;
    for (int k = 0; k < 8; ++k) P.sr[k] = rr ? (float)(g.coefr[k] * std::pow(pikr * pikr, k)) : (k == 0 ? 1.f : 0.f);
    P.pikr2 = rr ? (float)(pikr * pikr) : 0.f;
    P.e21 = (float)(dp.eps2 / dp.eps1);
    P.s2tir = (float)(std::sin(1e4) * std::sin(1e4));
    P.t0rec = nullptr; P.tq0 = nullptr;
    return P;
}

// Arguments of the ttype-0 pair kernel: targets [ntl1, ntl) of each trace.
// genRefrPhasor's path applies fEI and fEO (attenuation, roughness,
// reradiation) whatever `lossless` says (sim.cu:940-966).
PairArgs seg_pair_args_t0(const Seg& g) {
    const DevParams& dp = g.sc->dp;
    PairArgs P = seg_pair_args(g);
    P.ntl = g.ntl; P.tq0 = g.ntl1; P.t0rec = g.t0rec;
    P.lossless = 0;
    P.ealpha = (float)(-2.0 * dp.alpha2 * 1.4426950408889634);
    P.eks = (float)(-2.0 * dp.ks * dp.ks * 1.4426950408889634);
    const double pikr = RP_PI * dp.fs / dp.lam;
    for (int k = 0; k < 8; ++k) P.sr[k] = (float)(g.coefr[k] * std::pow(pikr * pikr, k));
    P.pikr2 = (float)(pikr * pikr);
    const double kb0 = dp.c1_over_c2 / dp.dr, kt0 = 2.0 * dp.turn * dp.c1_over_c2;
    P.kb0 = (float)kb0;
    P.kb0h = (float)kb0; P.kb0l = (float)(kb0 - (double)P.kb0h);
    P.kt0h = (float)kt0; P.kt0l = (float)(kt0 - (double)P.kt0h);
    P.kr0 = (float)(2.0 * RP_PI * kt0);
    // rerad_funct (radar_kernels.cu:167-189) as a test on cos(TargetTh):
    // 1 and 2 keep angles below 1 and 0.5 degree, 3 below 3 * 180 / pi_F
    // radians (the reference's unit slip), 4 a Gaussian of width 1 degree
    const int f = dp.rerad_funct;
    P.rf = (f >= 1 && f <= 4) ? f : 0;
    const double th0 = f == 1 ? RP_PI_F / 180 : (f == 2 ? 0.5 * RP_PI_F / 180 : 3 * 180 / RP_PI_F);
    P.rcos = th0 >= RP_PI ? -2.f : (float)std::cos(th0);
    const double sg = RP_PI_F / 180;
    P.rgl = (float)(-0.5 * 1.4426950408889634 / (sg * sg));
    return P;
}

ConvArgs seg_conv_args(const Seg& g) {
    const rp_scene* sc = g.sc;
    const int nr = sc->nr;
    ConvArgs C;
    C.ntl = g.ntl1; C.tstride = g.L.tstride; C.nb = g.nb; C.bt0 = g.bt0; C.T = g.T; C.T2 = g.T2; C.Wt = g.Wt;
    C.C2s = (const Cplx<float>*)sc->d_C2S; C.Hs = (const Cplx<float>*)sc->d_HS;
    C.nr = nr; C.n2 = 2 * nr; C.N = 2 * nr - 1; C.M = sc->mS;
    C.crop_K = sc->crop_K; C.crop_all = sc->crop_all;
    C.sig_scale = (float)(-1.0 / std::sqrt(sc->dp.P));
    C.part = g.part; C.nsplit = g.nsplit; C.work = nullptr;
    return C;
}

// The single-batch pair kernel of one segment in configuration cfg.
int launch_pairs_one(const Seg& g, unsigned int* work, int cfg, int sms, cudaStream_t st) {
    const size_t pair_smem = pair_smem_bytes(RP_WIN_WIDE);
    PairArgs P = seg_pair_args(g);
    P.work = work;
    void (*pk)(const PairArgs) = pick_pair_kernel(g.deg, cfg, g.sc->ortho != 0, g.sub > 1);
    if (int rc = rp_allow_dyn_smem((const void*)pk, pair_smem)) return rc;
    int occ = 0;
    RP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pk, RP_PAIR_THREADS, pair_smem));
    const int64_t items = ((int64_t)g.nb * P.tblocks) << P.lparts;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)std::max(occ, 1) * sms, items));
    pk<<<grid, RP_PAIR_THREADS, pair_smem, st>>>(P);
    return RP_OK;
}

// Pair launch of a wave: the single-batch kernel (constants in the parameter
// bank) for one segment; for several, the multi-job kernel (cfg 0-3), one
// single-batch kernel per segment (cfg 4-7: configuration cfg - 4, on the
// workspace's auxiliary streams when par), or one per-kind multi-job kernel
// per (sinc degree, frame kind) group with the jobs in the parameter space
// (cfg 8-9).  The multi-job kernel's 10-way dispatch makes it spill; the
// other two read their constants from the parameter bank.  seg_work: one
// work counter per segment of ps; h_jobs: the job table on the host.
int launch_pairs(const std::vector<Seg*>& ps, const PairJob* d_jobs, const PairJob* h_jobs,
                 const unsigned int* d_start, unsigned int* d_work, unsigned int* seg_work, int cfg, int sms,
                 cudaStream_t st, rp_workspace* ws, bool par) {
    if (ps.size() > 1 && cfg >= 8) {
        // the (sinc degree, frame kind) groups' launches run concurrently on
        // the auxiliary streams, so one group's tail overlaps another's work
        if (par) ws->fork(st);
        const int rc = par ? launch_pairs_multik(cfg - 8, h_jobs, (int)ps.size(), seg_work, sms, st, ws->aux,
                                                 rp_workspace::kAux)
                           : launch_pairs_multik(cfg - 8, h_jobs, (int)ps.size(), seg_work, sms, st);
        if (par) ws->join(st);
        if (rc) return rc;
        RP_LAUNCHED();
        return RP_OK;
    }
    if (ps.size() > 1 && cfg >= 4) {
        // segments by decreasing work (items x facet-part capacity x targets
        // per block), dealt round robin to the auxiliary streams: each
        // stream's last launches are its short ones
        std::vector<size_t> order(ps.size());
        std::vector<double> work(ps.size());
        for (size_t i = 0; i < ps.size(); ++i) {
            const Seg& g = *ps[i];
            const double tb = (double)((g.L.tstride + RP_PAIR_THREADS - 1) / RP_PAIR_THREADS);
            work[i] = (double)g.nb * tb * (double)g.L.rstride * (double)std::min<int64_t>(g.L.tstride, RP_PAIR_THREADS);
            order[i] = i;
        }
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return work[a] > work[b]; });
        if (par) ws->fork(st);
        for (size_t k = 0; k < order.size(); ++k) {
            const size_t i = order[k];
            const cudaStream_t ss = par ? ws->aux[k % rp_workspace::kAux] : st;
            if (int rc = launch_pairs_one(*ps[i], seg_work + i, cfg - 4, sms, ss)) return rc;
            RP_LAUNCHED();
        }
        if (par) ws->join(st);
        return RP_OK;
    }
    if (ps.size() == 1 && ps[0]->sc->dp.specular) {     // specular waves hold one segment
        const Seg& g = *ps[0];
        PairArgs P = seg_pair_args(g);
        P.work = d_work;
        const int64_t items = (int64_t)g.nb * P.tblocks * RP_PARTS;
        if (int rc = launch_pairs_spec(g.deg, cfg, P, items, sms, st)) return rc;
    } else if (ps.size() == 1) {
        if (int rc = launch_pairs_one(*ps[0], d_work, cfg, sms, st)) return rc;
    } else {
        int64_t items = 0;
        for (const Seg* g : ps) items += (int64_t)g->nb * ((g->L.tstride + RP_PAIR_THREADS - 1) / RP_PAIR_THREADS) * RP_PARTS;
        const int rc = launch_pairs_multi(cfg, d_jobs, d_start, (int)ps.size(), d_work, items, sms, st);
        if (rc) return rc;
    }
    RP_LAUNCHED();
    return RP_OK;
}

// Zero the pair-stage outputs of a wave (T windows, work counters, flags).
int zero_pairs(const std::vector<Seg*>& ps, unsigned int* d_work, unsigned int* seg_work, cudaStream_t st) {
    for (const Seg* g : ps) {
        RP_CUDA(cudaMemsetAsync(g->T, 0, sizeof(C32) * 2 * g->row_elems(), st));
        if (g->T2) RP_CUDA(cudaMemsetAsync(g->T2, 0, sizeof(C32) * 2 * g->row_elems(), st));
        RP_CUDA(cudaMemsetAsync(g->misc + 1, 0, sizeof(int) * 3, st));
    }
    RP_CUDA(cudaMemsetAsync(d_work, 0, sizeof(unsigned int), st));
    RP_CUDA(cudaMemsetAsync(seg_work, 0, sizeof(unsigned int) * ps.size(), st));
    return RP_OK;
}

// Choose the pair configuration of a wave: the tuned one, or probe every
// candidate (four for one segment, two for the specular kernel, ten for a
// multi-segment wave: the multi-job kernel, per-segment launches and the
// per-kind kernels); each probe is a full launch on this wave's items,
// outputs re-zeroed after, and every candidate is probed twice (the best of
// its two times counts).  Tuned per kind: single kernel (0), multi-segment
// (1) or specular (2), and sinc degree.
// Facet sub-splits per part for a wave of one segment (default mode,
// ttype-1 targets only).  A small call's items, traces x target blocks x
// RP_PARTS, can leave most of the pair kernel's resident blocks idle (one
// trace of a 36-block scene: 144 items for 304 blocks); splitting each
// part's facet range sub ways, into rows of their own that k_fold_parts
// adds back into the parts, spreads the call over them.  sub doubles while
// the items still fit one round of the slots, each sub-part keeps at least
// two chunks of facets and the extra rows stay under 1 GiB.
const int64_t kSubBytes = (int64_t)1 << 30;
std::atomic<int> g_split_parts{1};      // rp_split_parts

int pair_sub(const Seg& g, int slots) {
    const rp_scene* sc = g.sc;
    const FastLayout& L = g.L;
    if (!g_split_parts.load() || sc->dp.specular || sc->nt1 < sc->nt) return 1;
    const int64_t tblocks = (L.tstride + RP_PAIR_THREADS - 1) / RP_PAIR_THREADS;
    const int64_t items = (int64_t)L.nb * tblocks * RP_PARTS;
    // the row cap takes the host bound of the window width where the call
    // has one (the width a graph replay lays out), so that a direct call and
    // a replay of the same traces split alike and sum in the same order
    const int64_t wb = std::max<int64_t>(L.Wt, std::max(1, std::min(sc->nr, (g.wmax + 3) & ~3)));
    const int64_t part_bytes = (int64_t)2 * RP_PARTS * L.nb * L.tstride * wb * (int64_t)sizeof(C32);
    int sub = 1;
    while (sub < 32 && items * sub * 2 <= slots && L.mstride >= (int64_t)RP_PARTS * sub * 4 &&
           part_bytes * (2 * sub - 1) <= kSubBytes)
        sub *= 2;
    return sub;
}

// Upper bound of pair_sub's extra row bytes for a one-segment call laid out
// as L, whose window width is a bound of the one the call will measure.
int64_t pair_sub_bound_bytes(const rp_scene* sc, const FastLayout& L, int slots) {
    if (!g_split_parts.load() || sc->dp.specular || sc->nt1 < sc->nt) return 0;
    const int64_t tblocks = (L.tstride + RP_PAIR_THREADS - 1) / RP_PAIR_THREADS;
    if ((int64_t)L.nb * tblocks * RP_PARTS * 2 > slots || L.mstride < (int64_t)RP_PARTS * 4) return 0;
    const int64_t part_bytes = (int64_t)2 * RP_PARTS * L.nb * L.tstride * L.Wt * (int64_t)sizeof(C32);
    return std::min<int64_t>(kSubBytes, part_bytes * 31);
}

int choose_cfg(const std::vector<Seg*>& ps, const PairJob* d_jobs, const PairJob* h_jobs,
               const unsigned int* d_start, unsigned int* d_work, unsigned int* seg_work, int sms, cudaStream_t st,
               rp_workspace* ws, bool par, int* cfg_out) {
    const bool spec = ps.size() == 1 && ps[0]->sc->dp.specular;
    const int multi = spec ? 2 : (ps.size() > 1 ? 1 : 0);
    const int deg = multi == 1 ? -1 : ps[0]->deg;
    const int ncfg = spec ? 2 : (multi == 1 ? 10 : 4);
    // a scene in the stalled-copy test mode never tunes: its launches time out
    if (!autotune_on() || ps[0]->sc->stall_copies) {
        const int c = ps[0]->sc->pair_cfg;
        *cfg_out = spec ? (c & 1) : (multi == 1 ? c : (c & 3));
        return RP_OK;
    }
    int c = tuned_lookup(multi, deg);
    if (c >= 0) { *cfg_out = c; return RP_OK; }
    // no probes under capture (the warm-up call tuned), nor for a wave of
    // split parts (one kernel shape whatever the configuration; tuning
    // waits for a call that can tell the configurations apart)
    if (ws->graph_mode == 2 || (multi == 0 && ps[0]->sub > 1)) {
        const int d = ps[0]->sc->pair_cfg;
        *cfg_out = spec ? (d & 1) : (multi == 1 ? d : (d & 3));
        return RP_OK;
    }
    cudaEvent_t e0, e1;
    RP_CUDA(cudaEventCreate(&e0));
    RP_CUDA(cudaEventCreate(&e1));
    // two rounds (forward, then backward), each configuration's best time:
    // one probe per configuration let a noisy probe decide for the process
    std::vector<float> tbest(ncfg, 1e30f);
    int rc = RP_OK;
    for (int r = 0; r < 2 * ncfg && rc == RP_OK; ++r) {
        const int k = r < ncfg ? r : 2 * ncfg - 1 - r;
        rc = zero_pairs(ps, d_work, seg_work, st);
        cudaError_t e = rc ? cudaSuccess : cudaEventRecord(e0, st);
        if (!rc && e == cudaSuccess) rc = launch_pairs(ps, d_jobs, h_jobs, d_start, d_work, seg_work, k, sms, st, ws, par);
        if (!rc && e == cudaSuccess) e = cudaEventRecord(e1, st);
        if (!rc && e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (!rc && e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (!rc && e != cudaSuccess) rc = rp_cuda_fail(e, "autotune probe");
        if (!rc) tbest[k] = std::min(tbest[k], ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    // the default configuration unless another is at least 1% faster (the
    // probes' run-to-run spread is about that, and a near tie that flips
    // the choice costs as much as it gains)
    const int defc = spec ? (ps[0]->sc->pair_cfg & 1) : (ps[0]->sc->pair_cfg & 3);
    int bestc = defc;
    for (int k = 0; k < ncfg; ++k)
        if (tbest[k] < tbest[bestc]) bestc = k;
    if (tbest[bestc] > 0.99f * tbest[defc]) bestc = defc;
    tuned_store(multi, deg, bestc);
    *cfg_out = bestc;
    return zero_pairs(ps, d_work, seg_work, st);
}

int run_wave(std::vector<Seg>& segs, rp_workspace* ws, cudaStream_t st) {
    const int nseg = (int)segs.size();
    const int sms = segs[0].sc->sm_count;
    // ---- setup stage for every segment
    const bool capturing = ws->graph_mode == 2;
    {
        size_t need = 0;
        for (Seg& g : segs) need += seg_setup_bytes(g.sc, g.Lw);
        if (capturing && need > ws->arena.cap) {
            rp_set_error("graph capture: the setup buffers outgrew the warm-up call's");
            return RP_ERR_INTERNAL;
        }
        int rc = ws->arena.reserve(need);
        if (rc) return rc;
    }
    Arena& a = ws->arena;
    a.reset();
    g_timer.mark(0, st);
    // independent segments: their setup chains run concurrently on the
    // workspace's auxiliary streams (buffers are disjoint arena slices)
    const bool par = nseg > 1 && ws->ensure_aux() == RP_OK;
    if (par) {
        ws->fork(st);
        for (int i = 0; i < nseg; ++i) seg_setup(segs[i], a, ws->aux[i % rp_workspace::kAux]);
        ws->join(st);
    } else {
        for (Seg& g : segs) seg_setup(g, a, st);
    }
    RP_CUDA(cudaGetLastError());
    std::vector<int> h_misc(8 * (size_t)nseg, 0);
    if (!capturing) {
        for (int i = 0; i < nseg; ++i)
            RP_CUDA(cudaMemcpyAsync(&h_misc[8 * i], segs[i].misc, sizeof(int) * 8, cudaMemcpyDeviceToHost, st));
        g_timer.mark(1, st);
        RP_CUDA(cudaStreamSynchronize(st));
        g_timer.collect(0, 1);
        for (int i = 0; i < nseg; ++i)
            if (h_misc[8 * i + 6]) {
                rp_set_error("fast form: an illuminated-facet or target list exceeded its capacity");
                return RP_ERR_INTERNAL;
            }
    }
    // ---- pair-stage buffers and job tables
    std::vector<Seg*> ps, cs[3];
    size_t gslot[3] = {0, 0, 0};
    for (int i = 0; i < nseg; ++i) {
        Seg& g = segs[i];
        // the measured widest target window, or in graph mode the host bound
        // (a replay's traces are not known when the buffers are laid out)
        const int wt = ws->graph_mode ? g.wmax : h_misc[8 * i];
        g.Wt = std::max(1, std::min(g.sc->nr, (wt + 3) & ~3));
        g.L = fast_layout(g.sc, g.nb, g.tmax, g.Wt, g.fmax);
        g.cmode = conv_mode(g.sc);
        g.nsplit = (int)conv_splits(g.L.tstride);
        // specular mode without convolution has no pair or compression
        // stage: its direct sums (launch_direct) take the facets and pairs
        g.pairs = g.sc->nt > 0 && g.sc->nf > 0 && g.tmax > 0 && g.sc->dp.cmode != 2;
        if (g.pairs) ps.push_back(&g);
        if (g.pairs && g.cmode <= 2) {
            cs[g.cmode].push_back(&g);
            gslot[g.cmode] = std::max(gslot[g.cmode], conv_gslot(g.sc));
        }
    }
    if (nseg == 1 && ps.size() == 1) ps[0]->sub = pair_sub(*ps[0], 2 * sms);
    // one global compression scratch region per wave, shared by the mode-1
    // and mode-2 launches (they run one after the other on one stream)
    const size_t gscr_n = (size_t)sms * std::max(gslot[1], gslot[2]);
    const size_t ncs = cs[0].size() + cs[1].size() + cs[2].size();
    // compression job tables: one per (storage mode, length class), each
    // table's segments by decreasing transform length and target count (a
    // persistent launch then ends on short items)
    struct CGroup { int mode, nc; std::vector<Seg*> segs; };
    std::vector<CGroup> cg;
    for (int m = 0; m < 3; ++m)
        for (Seg* g : cs[m]) {
            const int nc = conv_length_class(m, 2 * g->sc->nr);
            size_t k = 0;
            while (k < cg.size() && !(cg[k].mode == m && cg[k].nc == nc)) ++k;
            if (k == cg.size()) cg.push_back(CGroup{m, nc, {}});
            cg[k].segs.push_back(g);
        }
    for (CGroup& G : cg)
        std::stable_sort(G.segs.begin(), G.segs.end(), [](const Seg* x, const Seg* y) {
            if (x->sc->nr != y->sc->nr) return x->sc->nr > y->sc->nr;
            return x->L.tstride > y->L.tstride;
        });
    {
        size_t need = 4096 + 1024 * (cg.size() + 1) + (ps.size() + ncs) * (sizeof(PairJob) + sizeof(ConvArgs) + 64)
                      + gscr_n * sizeof(C32);
        for (Seg& g : segs)
            need += seg_pair_bytes(g.sc, g.L) + (size_t)(g.sub - 1) * 2 * RP_PARTS * g.nb * g.L.tstride * g.Wt * sizeof(C32);
        if (capturing && need > ws->arena2.cap) {
            rp_set_error("graph capture: the pair-stage buffers outgrew the warm-up call's");
            return RP_ERR_INTERNAL;
        }
        int rc = ws->arena2.reserve(need);
        if (rc) return rc;
    }
    Arena& b = ws->arena2;
    b.reset();
    for (Seg& g : segs) {
        g.T = b.take<C32>((size_t)2 * g.row_elems());
        g.T2 = g.sc->dp.specular ? b.take<C32>((size_t)2 * g.row_elems()) : nullptr;
        g.dpart = g.sc->dp.cmode == 2 ? b.take<double2>((size_t)g.nb * RP_DS_GROUPS * g.sc->nr) : nullptr;
        if (g.t0rec) {
            g.sum0 = b.take<C32>((size_t)g.nb * g.sc->nr);
            g.r0 = b.take<C32>((size_t)g.nb * g.sc->nr);
            g.t0scr = b.take<C32>((size_t)g.nb * g.Lw.surf_slot);
            g.t0part = b.take<double2>((size_t)g.nb * RP_T0_GROUPS * g.sc->nr);
        }
        if (g.cmode <= 2) {
            g.part = b.take<C32>((size_t)g.nb * g.nsplit * 2 * g.sc->nr);
            g.tscr = trace_m_global(g.sc) ? b.take<C32>((size_t)g.nb * 4 * g.sc->nr) : nullptr;
        } else {
            g.Z = b.take<C32>((size_t)g.nb * g.L.tstride * g.sc->nr);
            g.cscr = b.take<C32>((size_t)g.L.slots * g.L.slot);
        }
    }
    C32* gscr = gscr_n ? b.take<C32>(gscr_n) : nullptr;
    // work counters: pairs, 3 compression modes, ttype-0 per segment, pairs per segment
    unsigned int* d_work = b.take<unsigned int>(4 + 2 * nseg);
    unsigned int* seg_work = d_work + 4 + nseg;
    PairJob* d_pjobs = b.take<PairJob>(std::max<size_t>(ps.size(), 1));
    unsigned int* d_pstart = b.take<unsigned int>(ps.size() + 1);
    std::vector<ConvArgs*> d_cjobs(cg.size());
    std::vector<unsigned int*> d_cstart(cg.size());
    for (size_t k = 0; k < cg.size(); ++k) {
        d_cjobs[k] = b.take<ConvArgs>(cg[k].segs.size());
        d_cstart[k] = b.take<unsigned int>(cg[k].segs.size() + 1);
    }
    unsigned int* d_cwork = b.take<unsigned int>(cg.size() + 1);     // compression work counters
    RP_CUDA(cudaMemsetAsync(d_work, 0, sizeof(unsigned int) * (4 + 2 * nseg), st));
    RP_CUDA(cudaMemsetAsync(d_cwork, 0, sizeof(unsigned int) * (cg.size() + 1), st));
    for (Seg& g : segs) {
        RP_CUDA(cudaMemsetAsync(g.T, 0, sizeof(C32) * 2 * g.row_elems(), st));
        if (g.T2) RP_CUDA(cudaMemsetAsync(g.T2, 0, sizeof(C32) * 2 * g.row_elems(), st));
    }
    std::vector<PairJob> hp;
    std::vector<unsigned int> hps(1, 0u);
    for (Seg* g : ps) {
        hp.push_back(PairJob{seg_pair_args(*g), g->deg, g->sc->ortho});
        hps.push_back(hps.back() + (unsigned)(g->nb * hp.back().a.tblocks * RP_PARTS));
    }
    std::vector<std::vector<ConvArgs>> hc(cg.size());
    std::vector<std::vector<unsigned int>> hcs(cg.size());
    std::vector<size_t> csm(cg.size(), 0);
    for (size_t k = 0; k < cg.size(); ++k) {
        const int m = cg[k].mode;
        hcs[k].assign(1, 0u);
        for (Seg* g : cg[k].segs) {
            hc[k].push_back(seg_conv_args(*g));
            hcs[k].push_back(hcs[k].back() + (unsigned)(g->nb * g->nsplit));
            // shared memory: X, W and U (mode 0), the working buffer (mode 1), the
            // sub-block buffer (mode 2)
            const size_t sx = m == 0 ? (size_t)(6 * g->sc->nr) : (m == 1 ? (size_t)(2 * g->sc->nr) : RP_CONV_CHUNK);
            csm[k] = std::max(csm[k], sx * sizeof(Cplx<float>));
        }
    }
    // host-to-device copies of the job tables; under capture from pinned
    // staging that lives as long as the graph (its copy nodes read it at
    // every replay)
    auto upload = [&](void* dst, const void* src, size_t bytes) -> int {
        if (!capturing) {
            RP_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
            return RP_OK;
        }
        void* h = ws->pin_take(bytes);
        if (!h) {
            rp_set_error("graph capture: pinned staging of %zu bytes exhausted", ws->pin_cap);
            return RP_ERR_BUDGET;
        }
        std::memcpy(h, src, bytes);
        RP_CUDA(cudaMemcpyAsync(dst, h, bytes, cudaMemcpyHostToDevice, st));
        return RP_OK;
    };
    if (!hp.empty()) {
        if (int rc = upload(d_pjobs, hp.data(), sizeof(PairJob) * hp.size())) return rc;
        if (int rc = upload(d_pstart, hps.data(), sizeof(unsigned int) * hps.size())) return rc;
    }
    for (size_t k = 0; k < cg.size(); ++k) {
        if (int rc = upload(d_cjobs[k], hc[k].data(), sizeof(ConvArgs) * hc[k].size())) return rc;
        if (int rc = upload(d_cstart[k], hcs[k].data(), sizeof(unsigned int) * hcs[k].size())) return rc;
    }
    // ---- pair stage: one launch for the wave
    if (!ps.empty()) {
        int cfg = 0;
        int rc = choose_cfg(ps, d_pjobs, hp.data(), d_pstart, d_work, seg_work, sms, st, ws, par, &cfg);
        if (rc) return rc;
        g_timer.mark(1, st);
        rc = launch_pairs(ps, d_pjobs, hp.data(), d_pstart, d_work, seg_work, cfg, sms, st, ws, par);
        if (rc) return rc;
        ++g_timer.pair_launches;
        // ttype-0 targets: one launch per segment that has them
        for (int i = 0; i < nseg; ++i) {
            Seg& g = segs[i];
            if (!g.pairs || !g.t0rec) continue;
            PairArgs P0 = seg_pair_args_t0(g);
            P0.work = d_work + 4 + i;
            const int64_t items = (int64_t)g.nb * P0.tblocks * RP_PARTS;
            rc = launch_pairs_t0(g.deg, g.sc->ortho != 0, g.sc->dp.specular != 0, P0, items, sms, st);
            if (rc) return rc;
            RP_LAUNCHED();
        }
        for (Seg* g : ps) {
            if (g->sub == 1) continue;
            const int64_t slot = (int64_t)g->nb * g->L.tstride * g->Wt;
            const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((slot + 255) / 256, (int64_t)8 * sms));
            k_fold_parts<<<grid, 256, 0, st>>>(reinterpret_cast<float4*>(g->T), slot, g->sub);
            RP_LAUNCHED();
        }
    } else {
        g_timer.mark(1, st);
    }
    g_timer.mark(2, st);
    // ---- range compression: one launch per job table (storage mode and
    // length class), the Bluestein kernel per segment whose nr is not a
    // power of two.  With several tables the mode-0 launches run on
    // auxiliary streams of their own, beside the mode-1 and mode-2 launches
    // on the last one (those share the global scratch, so they run in
    // turn), and each launch's tail overlaps the others' work.
    const bool cpar = cg.size() > 1 && ws->ensure_aux() == RP_OK;
    if (cpar) ws->fork(st);
    int n0 = 0;     // mode-0 launches so far
    for (size_t k = 0; k < cg.size(); ++k) {
        const int m = cg[k].mode;
        const cudaStream_t cst = !cpar ? st
                                       : (m == 0 ? ws->aux[(n0++) % (rp_workspace::kAux - 1)]
                                                 : ws->aux[rp_workspace::kAux - 1]);
        int rc = launch_conv32s(d_cjobs[k], d_cstart[k], (int)cg[k].segs.size(), m, cg[k].nc, csm[k], sms, sms,
                                hcs[k].back(), d_cwork + k, gscr, gslot[m], cg[k].segs[0]->sc->dp.specular != 0,
                                cst);
        if (rc) return rc;
    }
    if (cpar) ws->join(st);
    for (Seg* g : ps) {
        if (g->cmode <= 2) continue;
        const rp_scene* sc = g->sc;
        // the targets' chirp: the surface chirp in specular mode (sim.cu:851-856)
        k_conv32<<<g->L.slots, 256, 0, st>>>(g->ntl1, g->L.tstride, g->nb, g->bt0, g->T, g->T2, g->Wt, g->Z,
                                            (const C32*)(sc->dp.specular ? sc->d_C1_32 : sc->d_C2_32),
                                            plan_view32(sc->plan2), plan_view32(sc->planN),
                                            sc->crop_K, sc->crop_all, sc->nr, (float)(-1.0 / std::sqrt(sc->dp.P)),
                                            g->cscr, g->L.slot);
        RP_LAUNCHED();
    }
    RP_CUDA(cudaGetLastError());
    g_timer.mark(3, st);
    // ---- surface compression and the final sums (per segment; concurrent
    // on the auxiliary streams when the wave has several)
    if (par) ws->fork(st);
    for (int si = 0; si < nseg; ++si) {
        Seg& g = segs[si];
        const cudaStream_t ts = par ? ws->aux[si % rp_workspace::kAux] : st;
        const rp_scene* sc = g.sc;
        const int nr = sc->nr;
        if (g.dpart) {          // specular mode without convolution
            DirectArgs D;
            const DevParams& dp = sc->dp;
            D.F = sc->d_sorted; D.nf = std::max<int64_t>(sc->nf, 1); D.fstride = g.Lw.fstride; D.idx = g.idx; D.nill = g.nill; D.traces = g.trb;
            D.TG = sc->d_targets_fast; D.nt = sc->nt; D.tlist = g.tlist; D.ntl = g.ntl; D.tstride = g.Lw.tstride;
            D.sv = g.sv; D.spec = g.spec; D.t0rec = g.t0rec; D.rstride = g.Lw.rstride;
            D.PR = sc->d_prisms; D.np = sc->np; D.nr = nr;
            D.beta = dp.dr / dp.rng_res; D.inv_dr = dp.inv_dr; D.turn2 = 2.0 * dp.turn; D.c_c2 = dp.c_over_c2;
            D.alpha2 = dp.alpha2; D.ks2 = (float)(dp.ks * dp.ks);
            D.e21 = (float)(dp.eps2 / dp.eps1); D.s2tir = (float)(std::sin(1e4) * std::sin(1e4));
            const double pikr = RP_PI * dp.fs / dp.lam;
            D.pikr2 = (float)(pikr * pikr);
            const PairArgs R = seg_pair_args_t0(g);        // the rerad_funct test
            D.rf = R.rf; D.rcos = R.rcos; D.rgl = R.rgl;
            D.part = g.dpart;
            if (int rc = launch_direct(D, g.nb, g.d_out, g.out64, (int)g.s0, ts)) return rc;
            RP_LAUNCHED();
            continue;
        }
        const bool circ = sc->dp.cmode == 1;
        if (circ) {
            // specular with circular convolution: the reference's surface
            // convolution is commented out, so the surface is zero (sim.cu:765-767)
            RP_CUDA(cudaMemsetAsync(g.refl, 0, sizeof(C32) * g.nb * nr, ts));
        } else {
            // disable_surface has no effect in specular mode (sim.cu:740-772)
            k_surf_conv32<<<g.nb, 256, 0, ts>>>(g.acc, g.nill, g.vmax, sc->dp.specular ? 0 : sc->dp.disable_surface,
                                                nr, (const C32*)sc->d_C1_32, plan_view32(sc->plan2), g.refl, g.sscr,
                                                g.Lw.surf_slot);
            RP_LAUNCHED();
        }
        const C32* r0 = nullptr;
        if (g.pairs && g.t0rec) {      // ttype-0 targets: ordered sum, one chirp convolution per trace
            const size_t psm = (size_t)nr * sizeof(double2);
            const int use_smem = psm <= RP_T0_SMEM_MAX;
            if (use_smem) {
                if (int rc = rp_allow_dyn_smem((const void*)k_t0_part32, psm)) return rc;
            }
            k_t0_part32<<<dim3(RP_T0_GROUPS, g.nb), 256, use_smem ? psm : 0, ts>>>(
                g.ntl1, g.ntl, g.L.tstride, g.bt0, g.T, g.Wt, g.nb, nr, g.t0part, use_smem);
            RP_LAUNCHED();
            k_t0_sum32<<<dim3((nr + 255) / 256, g.nb), 256, 0, ts>>>(g.t0part, nr, g.sum0);
            RP_LAUNCHED();
            k_t0_conv32<<<g.nb, 256, 0, ts>>>(g.sum0, nr, (const C32*)(sc->dp.specular ? sc->d_C1_32 : sc->d_C2_32),
                                             plan_view32(sc->plan2), g.r0, g.t0scr, g.Lw.surf_slot, circ ? 1 : 0,
                                             (const C32*)sc->d_CR_32, circ ? plan_view32(sc->planR)
                                                                           : plan_view32(sc->plan2));
            RP_LAUNCHED();
            r0 = g.r0;
        }
        if (g.cmode <= 2) {
            if (!g.pairs) RP_CUDA(cudaMemsetAsync(g.part, 0, sizeof(C32) * g.nb * g.nsplit * 2 * nr, ts));
            const size_t tsm = g.tscr ? 0 : (size_t)4 * nr * sizeof(C32);
            if (int rc = rp_allow_dyn_smem((const void*)k_trace_m32, tsm)) return rc;
            k_usum32<<<dim3((2 * nr + 255) / 256, g.nb), 256, 0, ts>>>(g.nill, g.ntl1, g.part, g.nsplit, 2 * nr);
            RP_LAUNCHED();
            k_trace_m32<<<g.nb, 512, tsm, ts>>>(g.nill, g.ntl1, g.refl, g.part, g.nsplit, nr,
                                                 (const Cplx<float>*)sc->d_HS,
                                                 reinterpret_cast<Cplx<float>*>(g.tscr), g.d_out, g.out64,
                                                 (int)g.s0, r0);
        } else {
            if (!g.pairs) RP_CUDA(cudaMemsetAsync(g.Z, 0, sizeof(C32) * g.nb * g.L.tstride * nr, ts));
            k_sum32<<<dim3((nr + 255) / 256, g.nb), 256, 0, ts>>>(g.nill, g.ntl1, g.L.tstride, g.refl, g.Z, nr,
                                                                 g.d_out, g.out64, (int)g.s0, r0);
        }
        RP_LAUNCHED();
    }
    RP_CUDA(cudaGetLastError());    // before the join's event calls
    if (par) ws->join(st);
    if (capturing) {
        // flags and counts into pinned memory, read by rp_graph_check after
        // the replay has finished
        for (int i = 0; i < nseg; ++i) {
            int* hm = static_cast<int*>(ws->pin_take(sizeof(int) * 8));
            int* hc2 = static_cast<int*>(ws->pin_take(sizeof(int) * 2 * (size_t)segs[i].nb));
            if (!hm || !hc2) {
                rp_set_error("graph capture: pinned staging of %zu bytes exhausted", ws->pin_cap);
                return RP_ERR_BUDGET;
            }
            RP_CUDA(cudaMemcpyAsync(hm, segs[i].misc, sizeof(int) * 8, cudaMemcpyDeviceToHost, st));
            RP_CUDA(cudaMemcpyAsync(hc2, segs[i].nill, sizeof(int) * segs[i].nb, cudaMemcpyDeviceToHost, st));
            RP_CUDA(cudaMemcpyAsync(hc2 + segs[i].nb, segs[i].ntl, sizeof(int) * segs[i].nb, cudaMemcpyDeviceToHost,
                                    st));
            ws->graph_rb.push_back(rp_workspace::Readback{hm, hc2, segs[i].nb, segs[i].cbase + segs[i].s0});
        }
        return RP_OK;
    }
    g_timer.mark(4, st);
    std::vector<std::vector<int>> cnt(nseg);
    for (int i = 0; i < nseg; ++i)
        RP_CUDA(cudaMemcpyAsync(&h_misc[8 * i], segs[i].misc, sizeof(int) * 8, cudaMemcpyDeviceToHost, st));
    for (int i = 0; i < nseg; ++i) {
        if (!segs[i].h_counts) continue;
        cnt[i].resize(2 * (size_t)segs[i].nb);
        RP_CUDA(cudaMemcpyAsync(cnt[i].data(), segs[i].nill, sizeof(int) * segs[i].nb, cudaMemcpyDeviceToHost, st));
        RP_CUDA(cudaMemcpyAsync(cnt[i].data() + segs[i].nb, segs[i].ntl, sizeof(int) * segs[i].nb,
                                cudaMemcpyDeviceToHost, st));
    }
    RP_CUDA(cudaStreamSynchronize(st));
    g_timer.collect(1, 4);
    for (int i = 0; i < nseg; ++i) {
        if (h_misc[8 * i + 3]) { rp_set_error("fast form: a shared-memory stage wait timed out"); return RP_ERR_TIMEOUT; }
        if (h_misc[8 * i + 2]) { rp_set_error("fast form: a pair fell outside its target's bin window"); return RP_ERR_INTERNAL; }
    }
    for (int i = 0; i < nseg; ++i) {
        const Seg& g = segs[i];
        if (!g.h_counts) continue;
        for (int k = 0; k < g.nb; ++k) {
            g.h_counts[2 * (g.s0 + k)] = cnt[i][k];
            g.h_counts[2 * (g.s0 + k) + 1] = cnt[i][g.nb + k];
        }
    }
    return RP_OK;
}

std::vector<int> host_target_bounds(const rp_scene* sc, const double* tr, int64_t ns) {
    // An upper bound of each trace's in-aperture target count (k_target_flags
    // keeps acos(cos) <= aperture): cos >= cos(aperture + 1e-9) - 1e-9, tested
    // as (-r.v)^2 >= c0^2 |v|^2 without square roots or acos, so the bound is
    // a superset of the device's decision.  It sizes the segment's buffers
    // before any device work, so large calls split it over host threads.
    std::vector<int> ub(ns, 0);
    const int64_t nt = sc->nt;
    const double* tg = sc->h_targets.data();
    const double c0 = std::cos(sc->dp.ap_rad + 1e-9) - 1e-9;
    auto count = [&](int64_t s) {
        const double* r = tr + 9 * s;
        int c = 0;
        for (int64_t i = 0; i < nt; ++i) {
            const double vx = tg[i] - r[0], vy = tg[nt + i] - r[1], vz = tg[2 * nt + i] - r[2];
            const double d = -(r[3] * vx + r[4] * vy + r[5] * vz);
            const double m2 = vx * vx + vy * vy + vz * vz;
            const bool in = c0 > 0.0 ? (d > 0.0 && d * d >= c0 * c0 * m2) : (d >= c0 * std::sqrt(m2));
            c += in ? 1 : 0;
        }
        ub[s] = c;
    };
    const int64_t work = ns * nt;
    const int nth = (int)std::min<int64_t>(std::min<int64_t>(ns, 16), std::max<int64_t>(1, work / 200000));
    if (nth <= 1) {
        for (int64_t s = 0; s < ns; ++s) count(s);
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < nth; ++t)
            th.emplace_back([&, t] {
                for (int64_t s = t; s < ns; s += nth) count(s);
            });
        for (auto& x : th) x.join();
    }
    return ub;
}

// An upper bound of each trace's illuminated-facet count: the facets of the
// culling tiles whose bounding sphere is not wholly outside the aperture
// cone.  The test is the culling kernel's (tile_outside) with a margin of
// 1e-6 rad instead of 1e-9, so every tile the device keeps is counted here
// and the bound holds whatever the last-ulp differences of acos and asin
// between host and device.  It sizes the per-trace facet buffers (the
// illuminated list, the facet-pair records, the surface phasors) to the
// aperture's footprint instead of the whole store.  With wb, also a bound
// of each trace's target-window width for planning: k_tsetup32's window of a
// target spans (xmax - xmin) + kb (dmax - dmin) bins over the illuminated
// facets' bounding box, at most diag (1 + max(n, c1/c2)) / dr for the
// box's diagonal, here the diagonal of the kept tiles' box (plus margin).
std::vector<int64_t> host_facet_bounds(const rp_scene* sc, const double* tr, int64_t ns,
                                       std::vector<int>* wb = nullptr) {
    const int64_t nf = sc->nf;
    std::vector<int64_t> fb(ns, nf);
    if (wb) wb->assign(ns, sc->nr);
    const std::vector<double>& ts = sc->h_tiles_sorted;
    const int64_t ntl = (int64_t)ts.size() / 4;
    if (nf == 0 || ntl * RP_CULL_TILE < nf) return fb;
    const double ap = sc->dp.ap_rad;
    const double kw = (1.0 + std::max(sc->dp.nidx, sc->dp.c1_over_c2)) / sc->dp.dr;
    auto count = [&](int64_t s) {
        const double* r = tr + 9 * s;
        int64_t c = 0;
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int64_t t = 0; t < ntl; ++t) {
            const double* q = &ts[4 * t];
            const double vx = q[0] - r[0], vy = q[1] - r[1], vz = q[2] - r[2];
            const double d = std::sqrt(vx * vx + vy * vy + vz * vz);
            bool outside = false;
            if (d > q[3]) {
                const double cs = std::max(-1.0, std::min(1.0, -(vx * r[3] + vy * r[4] + vz * r[5]) / d));
                outside = std::acos(cs) - std::asin(q[3] / d) > ap + 1e-6;
            }
            if (!outside) {
                c += std::min<int64_t>(RP_CULL_TILE, nf - t * RP_CULL_TILE);
                for (int a = 0; a < 3; ++a) {
                    lo[a] = std::min(lo[a], q[a] - q[3]);
                    hi[a] = std::max(hi[a], q[a] + q[3]);
                }
            }
        }
        fb[s] = c;
        if (wb && c > 0) {
            double d2 = 0.0;
            for (int a = 0; a < 3; ++a) d2 += (hi[a] - lo[a]) * (hi[a] - lo[a]);
            const double w = std::ceil(std::sqrt(d2) * kw) + 8.0;
            (*wb)[s] = (int)std::min<double>((double)sc->nr, std::max(1.0, w));
        }
    };
    const int64_t work = ns * ntl;
    const int nth = (int)std::min<int64_t>(std::min<int64_t>(ns, 16), std::max<int64_t>(1, work / 50000));
    if (nth <= 1) {
        for (int64_t s = 0; s < ns; ++s) count(s);
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < nth; ++t)
            th.emplace_back([&, t] {
                for (int64_t s = t; s < ns; s += nth) count(s);
            });
        for (auto& x : th) x.join();
    }
    return fb;
}

// Size the next segment of a scene's traces starting at s0: up to 64 traces
// whose scratch (target windows bounded by nr, facet buffers by the traces'
// facet bounds fb) fits the budget.
void next_segment(const rp_scene* sc, const std::vector<int>& ub, const std::vector<int64_t>& fb,
                  const std::vector<int>& wb, int64_t s0, int64_t ns, int* nb_out, int64_t* tmax_out,
                  int64_t* fmax_out, size_t* bytes_out, int* wmax_out = nullptr) {
    int nb = 0;
    int64_t tmax = 0, fmax = 0;
    int wmax = 1;
    size_t bytes = 0;
    for (;;) {
        if (s0 + nb >= ns) break;
        const int64_t t2 = std::max<int64_t>(tmax, ub[s0 + nb]);
        const int64_t f2 = std::max<int64_t>(fmax, fb[s0 + nb]);
        const int w2 = std::max(wmax, wb[s0 + nb]);
        const FastLayout L = fast_layout(sc, nb + 1, t2, w2, f2);
        const size_t b2 = seg_setup_bytes(sc, L) + seg_pair_bytes(sc, L);
        if (nb > 0 && b2 > kFastBudget) break;
        tmax = t2;
        fmax = f2;
        wmax = w2;
        bytes = b2;
        ++nb;
        if (nb >= 64) break;
    }
    *nb_out = nb;
    *tmax_out = tmax;
    *fmax_out = fmax;
    *bytes_out = bytes;
    if (wmax_out) *wmax_out = wmax;
}

int check_scene(const rp_scene* sc) {
    // every mode rp_scene_create accepts runs here: the default mode,
    // specular with linear convolution, and specular with circular or no
    // convolution (ttype-0 targets only)
    if (sc->planN.pow2) { rp_set_error("internal: N = 2 nr - 1 is a power of two"); return RP_ERR_INTERNAL; }
    return RP_OK;
}

}  // namespace

// Peak scratch of a call: the largest wave of the same segment/wave plan the
// run makes (in-aperture target counts from the traces when given, else every
// target of the scene).
size_t rp_fast_plan_bytes(const rp_scene* sc, const double* h_traces, int64_t ns) {
    std::vector<int> ub = h_traces ? host_target_bounds(sc, h_traces, ns) : std::vector<int>(ns, (int)sc->nt);
    std::vector<int> wb(ns, sc->nr);
    std::vector<int64_t> fb = h_traces ? host_facet_bounds(sc, h_traces, ns, &wb) : std::vector<int64_t>(ns, sc->nf);
    size_t peak = 0, wave = 0;
    int nseg = 0;
    for (int64_t s0 = 0; s0 < ns; ++nseg) {
        int nb, wmax = 1;
        int64_t tmax, fmax;
        size_t bytes;
        next_segment(sc, ub, fb, wb, s0, ns, &nb, &tmax, &fmax, &bytes, &wmax);
        if (wave > 0 && (sc->dp.specular || wave + bytes > kFastBudget)) {     // specular: one segment a wave
            peak = std::max(peak, wave);
            wave = 0;
        }
        // a call of one segment may split its facet parts (pair_sub): the
        // extra rows, bounded with the segment's window bound
        if (s0 == 0 && nb >= ns)
            bytes += (size_t)pair_sub_bound_bytes(sc, fast_layout(sc, nb, tmax, wmax, fmax), 2 * sc->sm_count);
        wave += bytes;
        s0 += nb;
    }
    return std::max(peak, wave) + 4096;
}

size_t rp_fast_scratch(const rp_scene* sc, int64_t ns) { return rp_fast_plan_bytes(sc, nullptr, ns); }

// Splits every job into segments (<= 64 traces, scratch within the budget)
// and packs consecutive segments into waves under the same budget.
int rp_fast_batch(const rp_job* jobs, int njobs, rp_workspace* ws, cudaStream_t st) {
    std::vector<SceneConst> kc(njobs);
    std::vector<std::vector<double>> tr(njobs);
    // graph mode plans from the host copies of the jobs' traces (no device
    // readback: the call may be under stream capture)
    const bool host_plan = ws->graph_mode && (ws->plan_traces || !ws->plan_jobs.empty());
    if (host_plan && (ws->plan_jobs.empty() ? njobs != 1 : (int)ws->plan_jobs.size() != njobs)) {
        rp_set_error("graph capture: the planned traces do not match the call's jobs");
        return RP_ERR_INTERNAL;
    }
    for (int j = 0; j < njobs; ++j) {
        int rc = check_scene(jobs[j].scene);
        if (rc) return rc;
        kc[j] = scene_const(jobs[j].scene);
        tr[j].resize(9 * (size_t)jobs[j].ns);
        if (host_plan) {
            const double* h = ws->plan_jobs.empty() ? ws->plan_traces : ws->plan_jobs[j];
            std::copy(h, h + 9 * jobs[j].ns, tr[j].begin());
        }
        else if (jobs[j].ns)
            RP_CUDA(cudaMemcpyAsync(tr[j].data(), jobs[j].d_traces, sizeof(double) * 9 * jobs[j].ns,
                                    cudaMemcpyDeviceToHost, st));
    }
    if (!host_plan) RP_CUDA(cudaStreamSynchronize(st));
    std::vector<Seg> wave;
    size_t wave_bytes = 0;
    int64_t cbase = 0;      // the job's first trace over all jobs (graph readback)
    for (int j = 0; j < njobs; ++j) {
        rp_scene* sc = jobs[j].scene;
        const int64_t ns = jobs[j].ns;
        const int nr = sc->nr;
        std::vector<int> ub = host_target_bounds(sc, tr[j].data(), ns);
        std::vector<int> wb;
        std::vector<int64_t> fb = host_facet_bounds(sc, tr[j].data(), ns, &wb);
        for (int64_t s0 = 0; s0 < ns;) {
            int nb;
            int64_t tmax, fmax;
            size_t bytes;
            next_segment(sc, ub, fb, wb, s0, ns, &nb, &tmax, &fmax, &bytes);
            // a specular segment runs in a wave of its own (k_pairs32s is a
            // single-batch kernel)
            const bool alone = sc->dp.specular || (!wave.empty() && wave[0].sc->dp.specular);
            if (!wave.empty() && (alone || wave_bytes + bytes > kFastBudget)) {
                int rc = run_wave(wave, ws, st);
                if (rc) return rc;
                wave.clear();
                wave_bytes = 0;
            }
            Seg g;
            g.sc = sc;
            g.trb = jobs[j].d_traces + 9 * s0;
            g.s0 = s0;
            g.nb = nb;
            g.tmax = tmax;
            g.fmax = fmax;
            g.d_out = jobs[j].d_out;
            g.out64 = 0;
            g.h_counts = jobs[j].counts;
            g.deg = kc[j].deg;
            g.coef = kc[j].coef;
            g.coefr = kc[j].coefr;
            g.Lw = fast_layout(sc, nb, tmax, nr, fmax);
            for (int64_t k = s0; k < s0 + nb; ++k) g.wmax = std::max(g.wmax, wb[k]);
            g.cbase = cbase;
            wave.push_back(g);
            wave_bytes += bytes;
            s0 += nb;
        }
        cbase += ns;
    }
    if (!wave.empty()) {
        int rc = run_wave(wave, ws, st);
        if (rc) return rc;
    }
    return RP_OK;
}

int rp_fast_run(rp_scene* sc, rp_workspace* ws, const double* d_traces, int64_t ns, void* d_out, int out64,
                int64_t* h_counts, cudaStream_t st) {
    int rc = check_scene(sc);
    if (rc) return rc;
    if (!out64) {
        rp_job j{sc, d_traces, ns, d_out, h_counts};
        return rp_fast_batch(&j, 1, ws, st);
    }
    // complex128 output: same batches, out64 set on every segment
    std::vector<double> tr(9 * (size_t)ns);
    RP_CUDA(cudaMemcpyAsync(tr.data(), d_traces, sizeof(double) * 9 * ns, cudaMemcpyDeviceToHost, st));
    RP_CUDA(cudaStreamSynchronize(st));
    std::vector<int> ub = host_target_bounds(sc, tr.data(), ns);
    std::vector<int> wb;
    std::vector<int64_t> fb = host_facet_bounds(sc, tr.data(), ns, &wb);
    const SceneConst kc = scene_const(sc);
    for (int64_t s0 = 0; s0 < ns;) {
        int nb;
        int64_t tmax, fmax;
        size_t bytes;
        next_segment(sc, ub, fb, wb, s0, ns, &nb, &tmax, &fmax, &bytes);
        std::vector<Seg> w(1);
        Seg& g = w[0];
        g.sc = sc; g.trb = d_traces + 9 * s0; g.s0 = s0; g.nb = nb; g.tmax = tmax; g.fmax = fmax;
        g.d_out = d_out; g.out64 = 1; g.h_counts = h_counts; g.deg = kc.deg; g.coef = kc.coef; g.coefr = kc.coefr;
        g.Lw = fast_layout(sc, nb, tmax, sc->nr, fmax);
        rc = run_wave(w, ws, st);
        if (rc) return rc;
        s0 += nb;
    }
    return RP_OK;
}

extern "C" int rp_split_parts(int enable) {
    g_split_parts.store(enable ? 1 : 0);
    return RP_OK;
}

extern "C" int rp_autotune(int enable) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_autotune = enable ? 1 : 0;
    return RP_OK;
}

extern "C" int rp_autotune_query(int multi, int degree, int* cfg) {
    if (!cfg) { rp_set_error("rp_autotune_query: null cfg"); return RP_ERR_ARG; }
    const int kind = multi == 2 ? 2 : (multi ? 1 : 0);
    *cfg = tuned_lookup(kind, kind == 1 ? -1 : degree);
    return RP_OK;
}

extern "C" int rp_query_footprint_traces(const rp_scene* s, const double* traces, int64_t ns, int form,
                                         int64_t* bytes) {
    if (!s || !bytes || ns < 0 || (ns > 0 && !traces)) {
        rp_set_error("rp_query_footprint_traces: bad argument");
        return RP_ERR_ARG;
    }
    if ((form & 0xff) != RP_FORM_FAST_F32) return rp_query_footprint(s, ns, form, bytes);
    *bytes = (int64_t)rp_fast_plan_bytes(s, traces, ns);
    return RP_OK;
}
