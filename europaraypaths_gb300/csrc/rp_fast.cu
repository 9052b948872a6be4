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
#include <algorithm>
#include <cmath>
#include <vector>

#include "rp_common.cuh"
#include "rp_conv.cuh"

#define RP_CHUNK 256          // facets per chunk (one record tile)
#define RP_PAIR_THREADS 256   // targets per pair-kernel block
#define RP_WIN 16             // bins in a thread's per-chunk window
#define RP_PARTS 4            // facet-range splits per (trace, target block)
#define RP_SPIN_LIMIT (1 << 22)

namespace {

using C32 = Cx<float>;
using C64 = Cx<double>;

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

struct MinOp { __device__ double operator()(double a, double b) const { return fmin(a, b); } };
struct MaxOp { __device__ double operator()(double a, double b) const { return fmax(a, b); } };
struct MinOpF { __device__ float operator()(float a, float b) const { return fminf(a, b); } };
struct MaxOpF { __device__ float operator()(float a, float b) const { return fmaxf(a, b); } };

// ------------------------------------------------------ per-facet stage --
__global__ void __launch_bounds__(RP_CHUNK)
k_facets32(const double* __restrict__ F, int64_t nf, const int* __restrict__ idx,
           const int* __restrict__ nill, const double* __restrict__ traces, DevParams dp,
           FacetRec* __restrict__ rec, ChunkMeta* __restrict__ meta, int64_t rstride,
           int64_t mstride, float* __restrict__ sx_o, C32* __restrict__ sv_o,
           unsigned long long* __restrict__ vmax) {
    __shared__ double shd[32];
    __shared__ float shf[32];
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
        i = idx[(size_t)s * nf + j];
        fx = F[i]; fy = F[nf + i]; fz = F[2 * nf + i];
    }
    // chunk bounding box and centre (FP64)
    double mnx = block_reduce(ok ? fx : 1e300, MinOp(), shd);
    double mny = block_reduce(ok ? fy : 1e300, MinOp(), shd);
    double mnz = block_reduce(ok ? fz : 1e300, MinOp(), shd);
    double mxx = block_reduce(ok ? fx : -1e300, MaxOp(), shd);
    double mxy = block_reduce(ok ? fy : -1e300, MaxOp(), shd);
    double mxz = block_reduce(ok ? fz : -1e300, MaxOp(), shd);
    const double cx = 0.5 * (mnx + mxx), cy = 0.5 * (mny + mxy), cz = 0.5 * (mnz + mxz);
    float xI = 0.f, rr = 0.f;
    if (ok) {
        double dx = fx - t.sx, dy = fy - t.sy, dz = fz - t.sz;
        double d = sqrt(dx * dx + dy * dy + dz * dz);
        double Ix = dx / d, Iy = dy / d, Iz = dz / d;
        double nx = F[3 * nf + i], ny = F[4 * nf + i], nz = F[5 * nf + i];
        double ux = F[6 * nf + i], uy = F[7 * nf + i], uz = F[8 * nf + i];
        double vx = F[9 * nf + i], vy = F[10 * nf + i], vz = F[11 * nf + i];
        double th = acos(clamp1(-Ix * nx - Iy * ny - Iz * nz));
        double ph = atan2(Ix * ux + Iy * uy + Iz * uz, Ix * vx + Iy * vy + Iz * vz);
        double sR = sqrt(dp.eps1 / dp.eps2) * sin(th);
        double rth = sR > 1.0 ? 1e4 : asin(sR);
        double cI = cos(th), cR = cos(rth);
        double rho = (dp.nu2 * cI - dp.nu1 * cR) / (dp.nu2 * cI + dp.nu1 * cR);
        double frc = 1.0 - rho * rho;
        double fre = rho * rho;
        if (rth > 1e3) frc = 0.0;
        double atm = exp(-4.0 * dp.alpha1 * d);
        fre *= atm;
        frc *= atm;
        fre *= exp(-4 * ((dp.ks * cI) * (dp.ks * cI)));
        double G = d_facet_G(th, ph, dp.lam, dp.fs);
        // surface leg (surfacePT, radar_kernels.cu:714-764)
        double Pf = d_friis(dp.P, t.grefr, G, dp.lam, d);
        double Ps = d_friis(Pf, G, t.grefr, dp.lam, d);
        if (!dp.lossless) Ps *= fre;
        double amp = sqrt(Ps);
        // phase in turns: phasor(2 Itd) = exp(-j (2 pi_F/lam) 2 Itd) = exp(-j 2 pi tt)
        double tt = 2.0 * d * dp.turn;
        double ft = tt - floor(tt);
        double sn, cs;
        sincospi(-2.0 * ft, &sn, &cs);
        sx_o[(size_t)s * nf + j] = (float)((d - t.rst) / dp.dr);
        sv_o[(size_t)s * nf + j] = C32{(float)(amp * cs), (float)(amp * sn)};
        atomic_max_pos(vmax + s, amp);
        // hoisted target-leg amplitude: sqrt(P Gr G frc n) lam^2 Dmax / ((4 pi)^2 Itd)
        const double f4 = (4 * RP_PI_FRIIS) * (4 * RP_PI_FRIIS);
        const double Dmax = (4 * RP_PI_F * dp.fs * dp.fs) / (dp.lam * dp.lam);
        double Kf = sqrt(dp.P * t.grefr * G * (dp.lossless ? 1.0 : frc) * dp.nidx) * dp.lam *
                    dp.lam * Dmax / (f4 * d);
        xI = (float)((d - t.rst) / dp.dr);
        double ti = d * dp.turn;
        float tauI = (float)(ti - floor(ti));
        float ddx = (float)(fx - cx), ddy = (float)(fy - cy), ddz = (float)(fz - cz);
        rr = sqrtf(ddx * ddx + ddy * ddy + ddz * ddz);
        FacetRec r;
        r.a = make_float4(ddx, ddy, ddz, ddx * ddx + ddy * ddy + ddz * ddz);
        r.b = make_float4((float)nx, (float)ny, (float)nz, xI);
        r.c = make_float4((float)ux, (float)uy, (float)uz, tauI);
        r.d = make_float4((float)vx, (float)vy, (float)vz, (float)Kf);
        rec[(size_t)s * rstride + j] = r;
    }
    float R = block_reduce(ok ? rr : 0.f, MaxOpF(), shf);
    float xmn = block_reduce(ok ? xI : 3e38f, MinOpF(), shf);
    float xmx = block_reduce(ok ? xI : -3e38f, MaxOpF(), shf);
    if (threadIdx.x == 0) {
        ChunkMeta m;
        m.cx = cx; m.cy = cy; m.cz = cz;
        m.R = R * (1.0f + 1e-6f) + 1e-4f;
        m.xmin = xmn; m.xmax = xmx;
        m.n = min(RP_CHUNK, n - k * RP_CHUNK);
        m.bbmin[0] = mnx; m.bbmin[1] = mny; m.bbmin[2] = mnz;
        m.bbmax[0] = mxx; m.bbmax[1] = mxy; m.bbmax[2] = mxz;
        meta[(size_t)s * mstride + k] = m;
    }
}

// Fixed-point accumulation of the surface leg (same scheme as the plain form).
__global__ void k_surf_fix32(int64_t nf, const int* __restrict__ nill, const float* __restrict__ sx,
                             const C32* __restrict__ sv, const unsigned long long* __restrict__ vmax,
                             int nr, long long* __restrict__ acc) {
    const int s = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = nill[s];
    if (j >= n) return;
    double vm = __longlong_as_double((long long)vmax[s]);
    if (!(vm > 0)) return;
    const double scale = ldexp(1.0, RP_FIX_BITS) / (2.0 * (double)n * vm);
    double x = sx[(size_t)s * nf + j];
    if (!(x > -1.0) || x >= (double)nr) return;
    long b = (long)x;
    double w = x - (double)b;
    C32 v = sv[(size_t)s * nf + j];
    long long* a = acc + (size_t)s * nr * 2;
    fix_add(a + 2 * b, (double)v.x * (1.0 - w), scale);
    fix_add(a + 2 * b + 1, (double)v.y * (1.0 - w), scale);
    if (b + 1 < nr) {
        fix_add(a + 2 * (b + 1), (double)v.x * w, scale);
        fix_add(a + 2 * (b + 1) + 1, (double)v.y * w, scale);
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
    const double kb = dp.nidx / dp.dr;
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
    float kb;           // n / dr
    float kt;           // n / lam
    float pik;          // pi * (pi_F * fs / lam): sinc arguments in radians
    float ealpha;       // -2 alpha2 log2(e)
    float eks;          // -2 ks^2 log2(e)
    double nidx, inv_dr, inv_lam;   // inv_lam: turns per metre, pi_F / (pi lam)
    int lossless;
};

__device__ __forceinline__ float sinc_rad(float a) {
    // sin(a)/a with a = pi x; 1 when |x| < 1e-6 (elementary_kernels.cu:50-53)
    return (fabsf(a) < 3.14159265e-6f) ? 1.0f : __sinf(a) / a;
}

__global__ void __launch_bounds__(RP_PAIR_THREADS)
k_pairs32(PairArgs A) {
    extern __shared__ __align__(128) unsigned char smem[];
    FacetRec* srec = reinterpret_cast<FacetRec*>(smem);                     // [2][RP_CHUNK]
    float2* win = reinterpret_cast<float2*>(smem + 2 * RP_CHUNK * sizeof(FacetRec));  // [RP_WIN][threads]
    __shared__ uint64_t bars[2];
    __shared__ unsigned int s_item;
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    uint32_t phase[2] = {0u, 0u};
    const unsigned int items = (unsigned)A.nb * A.tblocks * RP_PARTS;
    for (;;) {
        if (tid == 0) s_item = atomicAdd(A.work, 1u);
        __syncthreads();
        const unsigned int item = s_item;
        __syncthreads();
        if (item >= items) break;
        const int part = item % RP_PARTS;
        const int tb = (item / RP_PARTS) % A.tblocks;
        const int s = item / (RP_PARTS * A.tblocks);
        const int nq = A.ntl[s];
        const int n = A.nill[s];
        if (tb * RP_PAIR_THREADS >= nq || n == 0) continue;
        const int nchunks = (n + RP_CHUNK - 1) / RP_CHUNK;
        const int k0 = (int)((int64_t)nchunks * part / RP_PARTS);
        const int k1 = (int)((int64_t)nchunks * (part + 1) / RP_PARTS);
        if (k0 >= k1) continue;
        const int q = tb * RP_PAIR_THREADS + tid;
        const bool active = q < nq;
        double tx = 0, ty = 0, tz = 0;
        float tnx = 0, tny = 0, tnz = 1;
        int b0 = 0;
        C32* Trow = nullptr;
        if (active) {
            const int64_t ti = A.tlist[(size_t)s * A.tstride + q];
            tx = A.TG[ti]; ty = A.TG[A.nt + ti]; tz = A.TG[2 * A.nt + ti];
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
            const ChunkMeta m = A.meta[(size_t)s * A.mstride + k];
            if (!mbar_wait(&bars[buf], phase[buf])) {
                if (tid == 0) atomicOr(A.err + 1, 1u);
            }
            phase[buf] ^= 1u;
            const FacetRec* R = srec + buf * RP_CHUNK;
            if (active) {
                // FP64 anchors of this (chunk, target)
                const double Dx = tx - m.cx, Dy = ty - m.cy, Dz = tz - m.cz;
                const double T0 = sqrt(Dx * Dx + Dy * Dy + Dz * Dz);
                const double xt = A.nidx * T0 * A.inv_dr;
                const double tt = A.nidx * T0 * A.inv_lam;
                const float tau0 = (float)(tt - floor(tt));
                const float Dxf = (float)Dx, Dyf = (float)Dy, Dzf = (float)Dz;
                const float T0f = (float)T0;
                const float T0sq = (float)(T0 * T0);
                const double lo = (double)m.xmin + A.nidx * ((double)T0 - (double)m.R) * A.inv_dr;
                const int blo = (int)floor(lo) - 1;
                const float xbase = (float)(xt - (double)blo);     // x - blo = xI + xbase + kb dT
                for (int w = 0; w < RP_WIN; ++w) win[w * RP_PAIR_THREADS + tid] = make_float2(0.f, 0.f);
                const int cnt = m.n;
                for (int jj = 0; jj < cnt; ++jj) {
                    const FacetRec r = R[jj];
                    // d = target - facet = D - delta;  Ttd^2 - T0^2 = -2 D.delta + |delta|^2
                    const float dd = fmaf(Dxf, r.a.x, fmaf(Dyf, r.a.y, Dzf * r.a.z));
                    const float qd = fmaf(-2.f, dd, r.a.w);
                    const float d2 = T0sq + qd;
                    const float rinv = rsqrtf(d2);
                    const float Ttd = d2 * rinv;
                    const float dT = __fdividef(qd, Ttd + T0f);
                    const float jx = (Dxf - r.a.x) * rinv;
                    const float jy = (Dyf - r.a.y) * rinv;
                    const float jz = (Dzf - r.a.z) * rinv;
                    float cT = -fmaf(jx, r.b.x, fmaf(jy, r.b.y, jz * r.b.z));
                    float cD = -fmaf(jx, tnx, fmaf(jy, tny, jz * tnz));
                    cT = fminf(1.f, fmaxf(-1.f, cT));
                    cD = fminf(1.f, fmaxf(-1.f, cD));
                    const float yu = fmaf(jx, r.c.x, fmaf(jy, r.c.y, jz * r.c.z));
                    const float xv = fmaf(jx, r.d.x, fmaf(jy, r.d.y, jz * r.d.z));
                    const float h2 = fmaf(xv, xv, yu * yu);
                    const float aT = fmaf(-cT, cT, 1.f);
                    const float aD = fmaf(-cD, cD, 1.f);
                    // sin(th)cos(ph) = sqrt(a) xv / sqrt(h2); atan2(0,0) = 0 -> (sqrt(a), 0)
                    float g1, g2, g3, g4;
                    if (h2 > 0.f) {
                        const float gT = (aT > 0.f) ? aT * rsqrtf(aT * h2) : 0.f;
                        const float gD = (aD > 0.f) ? aD * rsqrtf(aD * h2) : 0.f;
                        g1 = gT * xv; g2 = gT * yu; g3 = gD * xv; g4 = gD * yu;
                    } else {
                        g1 = sqrtf(aT); g2 = 0.f; g3 = sqrtf(aD); g4 = 0.f;
                    }
                    const float S = sinc_rad(A.pik * g1) * sinc_rad(A.pik * g2) *
                                    sinc_rad(A.pik * g3) * sinc_rad(A.pik * g4);
                    float e2 = 0.f;
                    if (!A.lossless) {
                        float ea = A.ealpha * Ttd;
                        if (A.np > 0) {
                            // attenuation prisms (compTargetRays, geometry_kernels.cu:317-342)
                            const double fx = m.cx + r.a.x, fy = m.cy + r.a.y, fz = m.cz + r.a.z;
                            double tot = 0.0, ex = 0.0;
                            for (int64_t p = 0; p < A.np; ++p) {
                                double box[6] = {A.PR[A.np + p], A.PR[2 * A.np + p], A.PR[3 * A.np + p],
                                                 A.PR[4 * A.np + p], A.PR[5 * A.np + p], A.PR[6 * A.np + p]};
                                double ad = d_prism_dist(fx, fy, fz, jx, jy, jz, box, Ttd);
                                tot += ad;
                                ex += A.PR[p] * ad;
                            }
                            // ealpha = -2 alpha2 log2 e; the prism part replaces alpha2 there
                            ea = A.ealpha * (Ttd - (float)tot) - 2.f * 1.44269504f * (float)ex;
                        }
                        e2 = fmaf(A.eks, cT * cT, ea);
                    }
                    const float amp = r.d.w * fabsf(S) * rinv * exp2f(e2);
                    float tau = r.c.w + tau0 + A.kt * dT;
                    tau -= rintf(tau);
                    float sn, cs;
                    __sincosf(-6.28318530717958647f * tau, &sn, &cs);
                    const float vre = amp * cs, vim = amp * sn;
                    // bin of rngt: x = (Itd + n Ttd - rst)/dr, relative to blo
                    const float xr = r.b.w + xbase + A.kb * dT;     // x - blo
                    const float xabs = xr + (float)blo;
                    if (xabs > -1.f && xabs < A.nr_f) {
                        int b = (int)xabs;                            // truncation (short cast)
                        const float w = xabs - (float)b;
                        const int sl = b - blo;
                        const bool two = (b + 1) < A.nr;
                        if (sl >= 0 && sl + 1 < RP_WIN) {
                            float2* p0 = &win[sl * RP_PAIR_THREADS + tid];
                            float2 v0 = *p0;
                            v0.x = fmaf(vre, 1.f - w, v0.x);
                            v0.y = fmaf(vim, 1.f - w, v0.y);
                            *p0 = v0;
                            if (two) {
                                float2* p1 = p0 + RP_PAIR_THREADS;
                                float2 v1 = *p1;
                                v1.x = fmaf(vre, w, v1.x);
                                v1.y = fmaf(vim, w, v1.y);
                                *p1 = v1;
                            }
                        } else {
                            // outside the chunk window: direct update of the owned trace
                            const int o0 = b - b0;
                            if (o0 >= 0 && o0 < A.Wt) {
                                C32 t0 = Trow[o0];
                                t0.x = fmaf(vre, 1.f - w, t0.x);
                                t0.y = fmaf(vim, 1.f - w, t0.y);
                                Trow[o0] = t0;
                            } else {
                                atomicOr(A.err, 1u);
                            }
                            if (two) {
                                if (o0 + 1 >= 0 && o0 + 1 < A.Wt) {
                                    C32 t1 = Trow[o0 + 1];
                                    t1.x = fmaf(vre, w, t1.x);
                                    t1.y = fmaf(vim, w, t1.y);
                                    Trow[o0 + 1] = t1;
                                } else {
                                    atomicOr(A.err, 1u);
                                }
                            }
                        }
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
    if (tid == 0) {
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&bars[0])));
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&bars[1])));
    }
}

// ---------------------------------------------------------- compression --
// Per (trace, target): T = sum of the facet-range parts (fixed order) placed
// at its window; Ptarg = linconv(T, chirp2); contribution =
// convolveComplex(-T/sqrt(P), Ptarg) -> Z row (complex64, dense nr).
__global__ void k_conv32(const int* __restrict__ ntl, int64_t tstride, int nb, const int* __restrict__ bt0,
                         const C32* __restrict__ T, int Wt, C32* __restrict__ Z, const C32* __restrict__ C2,
                         PlanV<float> p2, PlanV<float> pN, int crop_K, int crop_all, int nr, float sig_scale,
                         C32* __restrict__ scratch, size_t slot) {
    C32* base = scratch + (size_t)blockIdx.x * slot;
    const int M = max(1 << p2.log2M, 1 << pN.log2M);
    C32* x = base;
    C32* wa = x + M;
    C32* wb = wa + M;
    C32* A = wb + M;
    C32* B = A + M;
    C32* tr = B + M;        // dense nr
    C32* ptarg = tr + nr;   // nr
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
                    const C32 u = T[(((size_t)p * nb + s) * tstride + q) * Wt + o];
                    v.x += u.x;
                    v.y += u.y;
                }
            }
            tr[i] = v;
        }
        __syncthreads();
        conv_linear_block<float>(tr, C2, p2, nr, x, wa, wb, ptarg, 1.0f);
        conv_complex_block<float>(tr, ptarg, pN, nr, crop_K, crop_all, A, B, wa, wb,
                                  Z + ((size_t)s * tstride + q) * nr, sig_scale);
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
                        void* __restrict__ out, int out64, int s0) {
    const int s = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nr) return;
    double vr = 0.0, vi = 0.0;
    if (nill[s] > 0) {
        C32 r = refl[(size_t)s * nr + i];
        vr = r.x; vi = r.y;
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
    int64_t rstride;     // records per trace (nf rounded to chunks)
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
    a.template take<unsigned long long>(L.nb);              // dmin
    a.template take<int>((size_t)L.nb * nf);                // idx
    a.template take<FacetRec>((size_t)L.nb * L.rstride);    // records
    a.template take<ChunkMeta>((size_t)L.nb * L.mstride);   // chunk meta
    a.template take<float>((size_t)L.nb * nf);              // surface x
    a.template take<C32>((size_t)L.nb * nf);                // surface v
    a.template take<TraceMeta>(L.nb);
    a.template take<uint8_t>((size_t)L.nb * nt);            // target flags
    a.template take<int>((size_t)L.nb * nt);                // tlist
    a.template take<int>((size_t)L.nb * L.tstride);         // bt0
    a.template take<int>(4);                                // maxw, work, err[2]
    a.template take<long long>((size_t)L.nb * nr * 2);      // surface fixed point
    a.template take<C32>((size_t)L.nb * nr);                // refl
    a.template take<C32>((size_t)L.nb * L.surf_slot);       // surface conv scratch
}

template <class Aa>
void fast_take_pairs(Aa& a, const rp_scene* sc, const FastLayout& L) {
    a.template take<C32>((size_t)RP_PARTS * L.nb * L.tstride * L.Wt);   // T parts
    a.template take<C32>((size_t)L.nb * L.tstride * sc->nr);            // Z
    a.template take<C32>((size_t)L.slots * L.slot);                      // conv scratch
}

FastLayout fast_layout(const rp_scene* sc, int nb, int64_t tstride, int Wt) {
    FastLayout L;
    L.nb = nb;
    L.tstride = std::max<int64_t>(tstride, 1);
    L.mstride = std::max<int64_t>((sc->nf + RP_CHUNK - 1) / RP_CHUNK, 1);
    L.rstride = L.mstride * RP_CHUNK;
    L.Wt = std::max(Wt, 1);
    const int M = std::max(sc->plan2.M(), sc->planN.M());
    L.slot = (size_t)5 * M + 2 * sc->nr;
    L.surf_slot = (size_t)3 * sc->plan2.M() + sc->nr;
    L.slots = std::max(1, 2 * sc->sm_count);
    return L;
}

const size_t kFastBudget = (size_t)32 << 30;

std::vector<int> host_target_bounds32(const rp_scene* sc, const std::vector<double>& tr, int64_t ns,
                                      const std::vector<double>& tg) {
    std::vector<int> ub(ns, 0);
    const int64_t nt = sc->nt;
    const double ap = sc->dp.ap_rad + 1e-9;
    for (int64_t s = 0; s < ns; ++s) {
        const double* r = &tr[9 * s];
        int c = 0;
        for (int64_t i = 0; i < nt; ++i) {
            double vx = tg[i] - r[0], vy = tg[nt + i] - r[1], vz = tg[2 * nt + i] - r[2];
            double m = std::sqrt(vx * vx + vy * vy + vz * vz);
            double cs = -r[3] * vx / m - r[4] * vy / m - r[5] * vz / m;
            cs = std::max(-1.0, std::min(1.0, cs));
            if (!(std::acos(cs) > ap)) ++c;
        }
        ub[s] = c;
    }
    return ub;
}

}  // namespace

size_t rp_fast_scratch(const rp_scene* sc, int64_t ns) {
    FastLayout L = fast_layout(sc, (int)std::max<int64_t>(1, std::min<int64_t>(ns, 16)), sc->nt, sc->nr);
    ArenaPlan a;
    fast_take_setup(a, sc, L);
    fast_take_pairs(a, sc, L);
    return a.off;
}

int rp_fast_run(rp_scene* sc, const double* d_traces, int64_t ns, void* d_out, int out64,
                int64_t* h_counts, cudaStream_t st) {
    const int64_t nf = sc->nf, nt = sc->nt;
    const int nr = sc->nr;
    if (sc->any_ttype0) {
        rp_set_error("fast form: ttype-0 targets are handled by the plain form only");
        return RP_ERR_UNSUPPORTED;
    }
    if (sc->planN.pow2) { rp_set_error("internal: N = 2 nr - 1 is a power of two"); return RP_ERR_INTERNAL; }
    std::vector<double> tr(9 * ns), tg(7 * nt);
    RP_CUDA(cudaMemcpyAsync(tr.data(), d_traces, sizeof(double) * 9 * ns, cudaMemcpyDeviceToHost, st));
    if (nt) RP_CUDA(cudaMemcpyAsync(tg.data(), sc->d_targets, sizeof(double) * 7 * nt, cudaMemcpyDeviceToHost, st));
    RP_CUDA(cudaStreamSynchronize(st));
    std::vector<int> ub = host_target_bounds32(sc, tr, ns, tg);
    PlanV<float> p2 = plan_view32(sc->plan2), pN = plan_view32(sc->planN);
    const DevParams& dp = sc->dp;
    const size_t pair_smem = 2 * RP_CHUNK * sizeof(FacetRec) + (size_t)RP_WIN * RP_PAIR_THREADS * sizeof(float2);
    RP_CUDA(cudaFuncSetAttribute(k_pairs32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pair_smem));
    int occ = 0;
    RP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_pairs32, RP_PAIR_THREADS, pair_smem));
    occ = std::max(occ, 1);
    for (int64_t s0 = 0; s0 < ns;) {
        int nb = 0;
        int64_t tmax = 0;
        for (;;) {
            if (s0 + nb >= ns) break;
            int64_t t2 = std::max<int64_t>(tmax, ub[s0 + nb]);
            FastLayout L = fast_layout(sc, nb + 1, t2, nr);
            ArenaPlan a;
            fast_take_setup(a, sc, L);
            fast_take_pairs(a, sc, L);
            if (nb > 0 && a.off > kFastBudget) break;
            tmax = t2;
            ++nb;
            if (nb >= 64) break;
        }
        // reserve for the worst window (Wt = nr) so no reallocation is needed
        FastLayout Lw = fast_layout(sc, nb, tmax, nr);
        {
            ArenaPlan a;
            fast_take_setup(a, sc, Lw);
            fast_take_pairs(a, sc, Lw);
            int rc = sc->arena.reserve(a.off);
            if (rc) return rc;
        }
        Arena& a = sc->arena;
        a.reset();
        const int64_t nfa = std::max<int64_t>(nf, 1), nta = std::max<int64_t>(nt, 1);
        const int tiles = (int)((std::max(nfa, nta) + RP_TILE - 1) / RP_TILE);
        uint8_t* fflags = a.take<uint8_t>((size_t)nb * nfa);
        int* tcnt = a.take<int>((size_t)nb * tiles);
        int* d_nill = a.take<int>(nb);
        int* d_ntl = a.take<int>(nb);
        unsigned long long* vmax = a.take<unsigned long long>(nb);
        unsigned long long* dmin = a.take<unsigned long long>(nb);
        int* idx = a.take<int>((size_t)nb * nfa);
        FacetRec* rec = a.take<FacetRec>((size_t)nb * Lw.rstride);
        ChunkMeta* meta = a.take<ChunkMeta>((size_t)nb * Lw.mstride);
        float* sxv = a.take<float>((size_t)nb * nfa);
        C32* sv = a.take<C32>((size_t)nb * nfa);
        TraceMeta* tm = a.take<TraceMeta>(nb);
        uint8_t* tflags = a.take<uint8_t>((size_t)nb * nta);
        int* tlist = a.take<int>((size_t)nb * nta);
        int* bt0 = a.take<int>((size_t)nb * Lw.tstride);
        int* misc = a.take<int>(4);
        long long* acc = a.take<long long>((size_t)nb * nr * 2);
        C32* refl = a.take<C32>((size_t)nb * nr);
        C32* sscr = a.take<C32>((size_t)nb * Lw.surf_slot);
        const double* trb = d_traces + 9 * s0;

        g_timer.mark(0, st);
        RP_CUDA(cudaMemsetAsync(vmax, 0, sizeof(unsigned long long) * nb, st));
        RP_CUDA(cudaMemsetAsync(dmin, 0xff, sizeof(unsigned long long) * nb, st));
        RP_CUDA(cudaMemsetAsync(acc, 0, sizeof(long long) * nb * nr * 2, st));
        RP_CUDA(cudaMemsetAsync(misc, 0, sizeof(int) * 4, st));
        if (nf > 0) {
            k_cull_count<<<dim3((unsigned)((nf + RP_TILE - 1) / RP_TILE), nb), RP_TILE_THREADS, 0, st>>>(
                sc->d_sorted, nf, trb, dp.ap_rad, fflags, tcnt, dmin);
            RP_LAUNCHED();
            compact_flags(fflags, nf, nb, tcnt, d_nill, idx, nfa, true, st);
            k_facets32<<<dim3((unsigned)Lw.mstride, nb), RP_CHUNK, 0, st>>>(
                sc->d_sorted, nfa, idx, d_nill, trb, dp, rec, meta, Lw.rstride, Lw.mstride, sxv, sv, vmax);
            RP_LAUNCHED();
            k_surf_fix32<<<dim3((unsigned)((nf + 255) / 256), nb), 256, 0, st>>>(nfa, d_nill, sxv, sv, vmax, nr, acc);
            RP_LAUNCHED();
            k_tmeta32<<<nb, 256, 0, st>>>(meta, Lw.mstride, d_nill, tm);
            RP_LAUNCHED();
        } else {
            RP_CUDA(cudaMemsetAsync(d_nill, 0, sizeof(int) * nb, st));
        }
        if (nt > 0) {
            k_target_flags<<<dim3((unsigned)((nt + 255) / 256), nb), 256, 0, st>>>(sc->d_targets, nt, trb,
                                                                                dp.ap_rad, tflags);
            RP_LAUNCHED();
            compact_flags(tflags, nt, nb, tcnt, d_ntl, tlist, Lw.tstride, false, st);
            if (nf > 0) {
                k_tsetup32<<<dim3((unsigned)((Lw.tstride + 255) / 256), nb), 256, 0, st>>>(
                    sc->d_targets, nt, tlist, d_ntl, Lw.tstride, tm, d_nill, dp, bt0, misc);
                RP_LAUNCHED();
            }
        } else {
            RP_CUDA(cudaMemsetAsync(d_ntl, 0, sizeof(int) * nb, st));
        }
        int h_maxw = 0;
        RP_CUDA(cudaMemcpyAsync(&h_maxw, misc, sizeof(int), cudaMemcpyDeviceToHost, st));
        g_timer.mark(1, st);
        RP_CUDA(cudaStreamSynchronize(st));
        g_timer.collect(0, 1);
        const int Wt = std::max(1, std::min(nr, (h_maxw + 3) & ~3));
        FastLayout L = fast_layout(sc, nb, tmax, Wt);
        C32* T = a.take<C32>((size_t)RP_PARTS * nb * L.tstride * Wt);
        C32* Z = a.take<C32>((size_t)nb * L.tstride * nr);
        C32* cscr = a.take<C32>((size_t)L.slots * L.slot);
        RP_CUDA(cudaMemsetAsync(T, 0, sizeof(C32) * RP_PARTS * nb * L.tstride * Wt, st));
        g_timer.mark(1, st);
        if (nt > 0 && nf > 0 && tmax > 0) {
            PairArgs P;
            P.rec = rec; P.meta = meta; P.rstride = Lw.rstride; P.mstride = Lw.mstride;
            P.nill = d_nill; P.ntl = d_ntl; P.tlist = tlist; P.tstride = L.tstride;
            P.TG = sc->d_targets; P.nt = nt; P.PR = sc->d_prisms; P.np = sc->np;
            P.bt0 = bt0; P.T = T; P.Wt = Wt; P.nb = nb;
            P.tblocks = (int)((L.tstride + RP_PAIR_THREADS - 1) / RP_PAIR_THREADS);
            P.work = reinterpret_cast<unsigned int*>(misc + 1);
            P.err = reinterpret_cast<unsigned int*>(misc + 2);
            P.nr_f = (float)nr; P.nr = nr;
            P.kb = (float)(dp.nidx / dp.dr);
            P.kt = (float)(dp.nidx * dp.turn);
            P.pik = (float)(RP_PI * (RP_PI_F * dp.fs / dp.lam));
            P.ealpha = (float)(-2.0 * dp.alpha2 * 1.4426950408889634);
            P.eks = (float)(-2.0 * dp.ks * dp.ks * 1.4426950408889634);
            P.nidx = dp.nidx; P.inv_dr = 1.0 / dp.dr; P.inv_lam = dp.turn;
            P.lossless = dp.lossless;
            int grid = std::min(occ * sc->sm_count, nb * P.tblocks * RP_PARTS);
            k_pairs32<<<grid, RP_PAIR_THREADS, pair_smem, st>>>(P);
            RP_LAUNCHED();
            ++g_timer.pair_launches;
            g_timer.mark(2, st);
            const float sig_scale = (float)(-1.0 / std::sqrt(dp.P));
            k_conv32<<<L.slots, 256, 0, st>>>(d_ntl, L.tstride, nb, bt0, T, Wt, Z, (const C32*)sc->d_C2_32,
                                             p2, pN, sc->crop_K, sc->crop_all, nr, sig_scale, cscr, L.slot);
            RP_LAUNCHED();
        }
        if (!(nt > 0 && nf > 0 && tmax > 0)) g_timer.mark(2, st);
        g_timer.mark(3, st);
        k_surf_conv32<<<nb, 256, 0, st>>>(acc, d_nill, vmax, dp.disable_surface, nr, (const C32*)sc->d_C1_32, p2,
                                         refl, sscr, Lw.surf_slot);
        RP_LAUNCHED();
        k_sum32<<<dim3((nr + 255) / 256, nb), 256, 0, st>>>(d_nill, d_ntl, L.tstride, refl, Z, nr, d_out, out64,
                                                           (int)s0);
        RP_LAUNCHED();
        g_timer.mark(4, st);
        RP_CUDA(cudaGetLastError());
        unsigned int herr[2] = {0, 0};
        std::vector<int> a1(nb), a2(nb);
        RP_CUDA(cudaMemcpyAsync(herr, misc + 2, sizeof(herr), cudaMemcpyDeviceToHost, st));
        RP_CUDA(cudaMemcpyAsync(a1.data(), d_nill, sizeof(int) * nb, cudaMemcpyDeviceToHost, st));
        RP_CUDA(cudaMemcpyAsync(a2.data(), d_ntl, sizeof(int) * nb, cudaMemcpyDeviceToHost, st));
        RP_CUDA(cudaStreamSynchronize(st));
        g_timer.collect(1, 4);
        if (herr[1]) { rp_set_error("fast form: a shared-memory stage wait timed out"); return RP_ERR_TIMEOUT; }
        if (herr[0]) { rp_set_error("fast form: a pair fell outside its target's bin window"); return RP_ERR_INTERNAL; }
        if (h_counts)
            for (int k = 0; k < nb; ++k) {
                h_counts[2 * (s0 + k)] = a1[k];
                h_counts[2 * (s0 + k) + 1] = a2[k];
            }
        s0 += nb;
    }
    return RP_OK;
}
