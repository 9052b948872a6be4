// rp_direct.cu -- the fast form of specular mode without convolution:
// reflRadarSignal and refrRadarSignal (radar_kernels.cu:58-299, sim.cu:
// 740-773, 940-986).  Per (trace, bin i) the reference sums over every
// illuminated facet j, and over every in-aperture target's (facet, target)
// pairs, w_j sinc((r_i - R_j) / res) with w_j = amplitude exp(+j 4 pi_F R_j
// / lam): a direct sum over facets x bins, kept here (no convolution
// exists to factor) but in FP32 on the tensor of sources x bins.
//
// With beta = dr / res and x_j = (R_j - rst) / dr, sinc(beta (i - x_j)) =
// [sin(pi beta i) cos(pi beta x_j) - cos(pi beta i) sin(pi beta x_j)] /
// (pi beta (i - x_j)): each source carries two complex weights c_j, s_j
// (w_j cos / sin(pi beta x_j) / (pi beta)) and a bin i adds c_j / (i - x_j)
// and s_j / (i - x_j) -- one reciprocal and four FMAs per (source, bin) --
// and multiplies the sums by sin(pi beta i), cos(pi beta i) once.  A source
// at |i - x_j| = d contributes terms of size |w| / (pi beta d) to the FP32
// sums, whose rounding then costs about 2 eps / (pi beta d) of |w| in the
// recombined bin: sources closer than RP_DS_NEAR (1/128 bin: at most ~2e-5
// of |w| beyond it) take the sinc directly instead.  The per-source
// geometry (ranges, phases) is FP64, amplitudes FP32.
#include <algorithm>

#include "rp_common.cuh"
#include "rp_internal.h"
#include "rp_pair.cuh"

namespace rpk {

namespace {

#define RP_DS_NEAR (1.f / 128.f)

// sin(pi beta x), cos(pi beta x) for a large x: exact reduction in FP64.
__device__ __forceinline__ void sincospi_bx(double bx, float& sp, float& cp) {
    const double m = rint(bx);
    const float f = (float)(bx - m);
    sincospif(f, &sp, &cp);
    if (((long long)m) & 1) { sp = -sp; cp = -cp; }
}

// One source's entry: x relative to the tile base, c and s, and w (near field).
__device__ __forceinline__ void ds_entry(double x, float wr, float wi, double base, const DirectArgs& A,
                                         float4& ea, float4& eb) {
    float sp, cp;
    sincospi_bx(A.beta * x, sp, cp);
    const float ip = (float)(1.0 / (RP_PI * A.beta));
    ea = make_float4((float)(x - base), wr * cp * ip, wi * cp * ip, wr * sp * ip);
    eb = make_float4(wi * sp * ip, wr, wi, 0.f);
}

// The thread's RP_DS_BPT bins (fi[b]: positions relative to the tile
// centre) take every staged entry; sums in FP32 over the block's facet
// group (its FP64 total is formed across groups).
__device__ __forceinline__ void ds_accumulate(const float4* sa, const float4* sb, const float* fi, float pib,
                                              float (*acc)[6]) {
#pragma unroll 2
    for (int k = 0; k < RP_DS_THREADS; ++k) {
        const float4 a = sa[k], b = sb[k];
        bool any_near = false;
        // far field, branch-free (the near bins get r = 0 here)
#pragma unroll
        for (int q = 0; q < RP_DS_BPT; ++q) {
            const float d = fi[q] - a.x;
            const bool near = fabsf(d) < RP_DS_NEAR;
            any_near |= near;
            const float r = near ? 0.f : rcp_a(d);
            acc[q][0] = fmaf(a.y, r, acc[q][0]);
            acc[q][1] = fmaf(a.z, r, acc[q][1]);
            acc[q][2] = fmaf(a.w, r, acc[q][2]);
            acc[q][3] = fmaf(b.x, r, acc[q][3]);
        }
        // the source's near bin (if any): the sinc itself
        if (__any_sync(0xffffffffu, any_near)) {
#pragma unroll
            for (int q = 0; q < RP_DS_BPT; ++q) {
                const float d = fi[q] - a.x;
                if (fabsf(d) < RP_DS_NEAR) {
                    const float z = pib * d;
                    const float sc = fabsf(z) < 3.14159265e-6f ? 1.f : __sinf(z) / z;
                    acc[q][4] = fmaf(b.y, sc, acc[q][4]);
                    acc[q][5] = fmaf(b.z, sc, acc[q][5]);
                }
            }
        }
    }
}

// Block (tile of RP_DS_TILE bins, facet group g, trace s); thread tid owns
// bins tile base + tid + k RP_DS_THREADS.  Each thread stages one facet of
// the chunk and evaluates that facet's sources: its surface phasor, then its
// pair with every in-aperture target in list order.
__global__ void __launch_bounds__(RP_DS_THREADS, 1) k_direct32(const __grid_constant__ DirectArgs A) {
    __shared__ float4 sa[RP_DS_THREADS], sb[RP_DS_THREADS];
    const int tile = blockIdx.x, g = blockIdx.y, s = blockIdx.z, tid = threadIdx.x;
    const int n = A.nill[s];
    // entries carry x relative to the tile centre (small, exact in FP32)
    const double base = (double)(tile * RP_DS_TILE + RP_DS_TILE / 2);
    float fi[RP_DS_BPT];
#pragma unroll
    for (int q = 0; q < RP_DS_BPT; ++q) fi[q] = (float)(tid + q * RP_DS_THREADS - RP_DS_TILE / 2);
    const float pib = (float)(RP_PI * A.beta);
    const TraceRow t = load_trace(A.traces, s);
    const int nq = A.ntl[s];
    float acc[RP_DS_BPT][6];
#pragma unroll
    for (int q = 0; q < RP_DS_BPT; ++q)
#pragma unroll
        for (int k = 0; k < 6; ++k) acc[q][k] = 0.f;
    const int nch = (n + RP_DS_THREADS - 1) / RP_DS_THREADS;
    const int c0 = (int)((int64_t)nch * g / RP_DS_GROUPS), c1 = (int)((int64_t)nch * (g + 1) / RP_DS_GROUPS);
    for (int c = c0; c < c1; ++c) {
        const int j = c * RP_DS_THREADS + tid;
        const bool ok = j < n;
        double fx = 0, fy = 0, fz = 0, itd = 0;
        float nx = 0, ny = 0, nz = 1, ux = 1, uy = 0, uz = 0, vx = 0, vy = 1, vz = 0;
        float sR = 0, cR = 1, cI = 1, sI = 0, a0 = 0;
        float4 ea = make_float4(1e30f, 0.f, 0.f, 0.f), eb = make_float4(0.f, 0.f, 0.f, 0.f);
        if (ok) {
            const int64_t f = A.idx[(size_t)s * A.fstride + j];
            const double* F = A.F;
            const int64_t m = A.nf;
            fx = F[f]; fy = F[m + f]; fz = F[2 * m + f];
            nx = (float)F[3 * m + f]; ny = (float)F[4 * m + f]; nz = (float)F[5 * m + f];
            ux = (float)F[6 * m + f]; uy = (float)F[7 * m + f]; uz = (float)F[8 * m + f];
            vx = (float)F[9 * m + f]; vy = (float)F[10 * m + f]; vz = (float)F[11 * m + f];
            const double dx = fx - t.sx, dy = fy - t.sy, dz = fz - t.sz;
            itd = sqrt(dx * dx + dy * dy + dz * dz);
            if (nq > 0) {           // the records exist when the scene has targets
                const size_t pj = ((size_t)s * A.rstride + j) >> 1;
                const int ln = j & 1;
                const FacetSpec sp = A.spec[pj];
                sR = ln ? sp.r.y : sp.r.x; cR = ln ? sp.r.w : sp.r.z;
                cI = ln ? sp.p.y : sp.p.x; sI = ln ? sp.p.w : sp.p.z;
                const float4 tv = A.t0rec[pj].v;
                a0 = ln ? tv.y : tv.x;
            }
            // reflRadarSignal's source: fRe exp(+j 4 pi_F Itd / lam) at Itd
            const C32 w = A.sv[(size_t)s * A.fstride + j];
            ds_entry((itd - t.rst) * A.inv_dr, w.x, w.y, base, A, ea, eb);
        }
        __syncthreads();            // the previous batch's entries are consumed
        sa[tid] = ea; sb[tid] = eb;
        __syncthreads();
        ds_accumulate(sa, sb, fi, pib, acc);
        for (int q = 0; q < nq; ++q) {
            // refrRadarSignal's source for (facet j, target q): rr = rerad(Tth)
            // fEI fEO radarEq(Itd + Ttd) at rngt = Itd + Ttd c/c2 (the plain
            // form's k_pairs64, geometry_kernels.cu:272-350, 520-584)
            ea = make_float4(1e30f, 0.f, 0.f, 0.f);
            eb = make_float4(0.f, 0.f, 0.f, 0.f);
            if (ok) {
                const int64_t ti = A.tlist[(size_t)s * A.tstride + q];
                const double ex = fx - A.TG[ti], ey = fy - A.TG[A.nt + ti], ez = fz - A.TG[2 * A.nt + ti];
                // Ttd from an FP32 reciprocal square root and one FP64 Newton step
                const double T2 = ex * ex + ey * ey + ez * ez;
                const float r0 = rsqrt_a((float)T2);
                const double rr0 = (double)r0;
                const double Ttd = T2 * rr0 * (1.5 - 0.5 * T2 * rr0 * rr0);
                const float rinv = r0;
                const float exf = (float)ex, eyf = (float)ey, ezf = (float)ez;
                const float pbr = (exf * nx + eyf * ny + ezf * nz) * rinv;     // cos Tth
                const float aT = fmaxf(0.f, 1.f - pbr * pbr);
                const float pc = exf * ux + eyf * uy + ezf * uz;
                const float pd = exf * vx + eyf * vy + ezf * vz - 1e-15f;      // atan2(0, 0) = 0
                const float rh = 1.f / (pc * pc + pd * pd);
                const float sTh = sqrtf(aT);
                const float st1 = sR * pbr - cR * sTh;
                const float q1 = st1 * st1;
                const float q2r = A.e21 * aT;
                const float q2 = q2r > 1.f ? A.s2tir : q2r;
                const float cn = cI * pd + sI * pc, sn = sI * pd - cI * pc;
                const float cc = cn * cn * rh, ss = sn * sn * rh;
                float num = 1.f, den = 1.f;
                sinc_sfu(q1 * cc * A.pikr2, num, den); sinc_sfu(q1 * ss * A.pikr2, num, den);
                sinc_sfu(q2 * cc * A.pikr2, num, den); sinc_sfu(q2 * ss * A.pikr2, num, den);
                const float gg = __fdividef(num, den);
                float rr = 1.f;
                if (A.rf >= 1 && A.rf <= 3) rr = pbr > A.rcos ? 1.f : 0.f;
                else if (A.rf == 4) {
                    const float th = acosf(fminf(1.f, fmaxf(-1.f, pbr)));
                    rr = exp2f(A.rgl * th * th);
                }
                double expo = A.alpha2 * Ttd;
                if (A.np > 0) {
                    const double jx = -ex / Ttd, jy = -ey / Ttd, jz = -ez / Ttd;
                    double tot = 0.0, ea2 = 0.0;
                    for (int64_t p = 0; p < A.np; ++p) {
                        double box[6] = {A.PR[A.np + p], A.PR[2 * A.np + p], A.PR[3 * A.np + p],
                                         A.PR[4 * A.np + p], A.PR[5 * A.np + p], A.PR[6 * A.np + p]};
                        const double ad = d_prism_dist(fx, fy, fz, jx, jy, jz, box, Ttd);
                        tot += ad;
                        ea2 += A.PR[p] * ad;
                    }
                    expo = ea2 + A.alpha2 * (Ttd - tot);
                }
                const float att2 = expf((float)(-8.0 * expo) - 8.f * A.ks2 * pbr * pbr);
                const float fri = (float)(1.0 / (itd + Ttd));
                const float f2 = fri * fri;
                const float amp = a0 * rr * gg * gg * att2 * (f2 * f2);
                const double rngt = itd + Ttd * A.c_c2;
                const double tt = A.turn2 * rngt;
                float sn2, cs2;
                sincospif(2.f * (float)(tt - rint(tt)), &sn2, &cs2);
                ds_entry((rngt - t.rst) * A.inv_dr, amp * cs2, amp * sn2, base, A, ea, eb);
            }
            __syncthreads();
            sa[tid] = ea; sb[tid] = eb;
            __syncthreads();
            ds_accumulate(sa, sb, fi, pib, acc);
        }
    }
#pragma unroll
    for (int q = 0; q < RP_DS_BPT; ++q) {
        const int i = tile * RP_DS_TILE + tid + q * RP_DS_THREADS;
        if (i < A.nr) {
            double sp, cp;
            sincospi(A.beta * (double)i, &sp, &cp);
            const double re = sp * acc[q][0] - cp * acc[q][2] + acc[q][4];
            const double im = sp * acc[q][1] - cp * acc[q][3] + acc[q][5];
            A.part[((size_t)s * RP_DS_GROUPS + g) * A.nr + i] = make_double2(re, im);
        }
    }
}

// The trace: the groups' partial sums in group order (FP64) -> output row s0 + s.
__global__ void k_direct_fin(const double2* __restrict__ part, int nr, void* __restrict__ out, int out64, int s0) {
    const int s = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nr) return;
    double vr = 0.0, vi = 0.0;
    for (int g = 0; g < RP_DS_GROUPS; ++g) {
        const double2 v = part[((size_t)s * RP_DS_GROUPS + g) * nr + i];
        vr += v.x;
        vi += v.y;
    }
    const size_t o = (size_t)(s0 + s) * nr + i;
    if (out64) reinterpret_cast<double2*>(out)[o] = make_double2(vr, vi);
    else reinterpret_cast<float2*>(out)[o] = make_float2((float)vr, (float)vi);
}

}  // namespace

int launch_direct(const DirectArgs& A, int nb, void* d_out, int out64, int s0, cudaStream_t st) {
    const dim3 grid((unsigned)((A.nr + RP_DS_TILE - 1) / RP_DS_TILE), RP_DS_GROUPS, (unsigned)nb);
    k_direct32<<<grid, RP_DS_THREADS, 0, st>>>(A);
    RP_CUDA(cudaGetLastError());
    k_direct_fin<<<dim3((unsigned)((A.nr + 255) / 256), (unsigned)nb), 256, 0, st>>>(A.part, A.nr, d_out, out64, s0);
    RP_CUDA(cudaGetLastError());
    return RP_OK;
}

}  // namespace rpk
