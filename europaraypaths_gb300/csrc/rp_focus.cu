// rp_focus.cu -- azimuth focusing of a radargram (src/PYTHON/simple_focusing.py),
// the processing step after the simulation:
//   * rp_focus_aperture: focus_rdrgrm (simple_focusing.py:310-404) -- every
//     pixel focused over its range row's synthetic aperture;
//   * rp_focus_center: full_focus_at_center (simple_focusing.py:115-185) --
//     range-cell-migration correction by integer rolls and one azimuth
//     matched filter for the whole image.
//
// The reference does both with FFTs in NumPy: per pixel (focus_rdrgrm) an FFT
// of length 2 * apt_smpl of which one sample is kept, per image an FFT of
// length 2 * Na along azimuth.  Each kept sample is one term of a circular
// convolution, so here every output is that convolution sum evaluated
// directly (FP32 complex, two accumulators), one thread per pixel.
//
// The per-row geometry of focus_rdrgrm is computed on the device with the
// IEEE operations NumPy performs, in its order (range, aperture, linspace,
// slant range, NumPy's float floor division), so the integer range-bin
// shifts equal the reference's bit for bit; the matched filter's refraction
// angle is a bracketed root (Brent's method) as the reference's brentq.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "rp_internal.h"

namespace {

// --------------------------------------------------------- FP64 geometry --
// NumPy's float floor division (npy_divmod): the quotient of a - fmod(a, b)
// by b, corrected toward the floor.
__device__ double np_floor_divide(double a, double b) {
    double mod = fmod(a, b);
    double div = __ddiv_rn(__dsub_rn(a, mod), b);
    if (mod != 0.0) {
        if ((b < 0) != (mod < 0)) div = __dsub_rn(div, 1.0);
    }
    double fl;
    if (div != 0.0) {
        fl = floor(div);
        if (__dsub_rn(div, fl) > 0.5) fl = __dadd_rn(fl, 1.0);
    } else {
        fl = copysign(0.0, __ddiv_rn(a, b));
    }
    return fl;
}

// refracted_angle (simple_focusing.py:82-86).
__device__ double refracted_angle(double th, double xoff, double h, double d, double sq_eps) {
    const double y = asin(sq_eps * sin(th));
    return h * tan(y) + d * tan(th) - xoff;
}

// Brent's method (R. P. Brent, Algorithms for Minimization without
// Derivatives, 1973, ch. 4) on [a, b]: inverse quadratic interpolation or
// secant steps inside the bracket, bisection when they stall; tolerance
// 2e-12 + 4 eps |x| as SciPy's brentq.  Returns false without a sign change.
__device__ bool brent(double xoff, double h, double d, double sq_eps, double a, double b, double* root) {
    double fa = refracted_angle(a, xoff, h, d, sq_eps), fb = refracted_angle(b, xoff, h, d, sq_eps);
    if (fa == 0.0) { *root = a; return true; }
    if (fb == 0.0) { *root = b; return true; }
    if ((fa > 0) == (fb > 0)) return false;
    double c = a, fc = fa, e = b - a, dd = e;
    for (int it = 0; it < 100; ++it) {
        if ((fb > 0) == (fc > 0)) { c = a; fc = fa; e = dd = b - a; }
        if (fabs(fc) < fabs(fb)) { a = b; b = c; c = a; fa = fb; fb = fc; fc = fa; }
        const double tol = 2e-12 + 4.0 * 2.220446049250313e-16 * fabs(b);
        const double m = 0.5 * (c - b);
        if (fabs(m) <= tol || fb == 0.0) break;
        if (fabs(e) >= tol && fabs(fa) > fabs(fb)) {
            double p, q, r;
            const double s = fb / fa;
            if (a == c) {
                p = 2.0 * m * s;
                q = 1.0 - s;
            } else {
                q = fa / fc;
                r = fb / fc;
                p = s * (2.0 * m * q * (q - r) - (b - a) * (r - 1.0));
                q = (q - 1.0) * (r - 1.0) * (s - 1.0);
            }
            if (p > 0) q = -q; else p = -p;
            if (2.0 * p < fmin(3.0 * m * q - fabs(tol * q), fabs(e * q))) {
                e = dd;
                dd = p / q;
            } else {
                dd = m;
                e = m;
            }
        } else {
            dd = m;
            e = m;
        }
        a = b;
        fa = fb;
        b += fabs(dd) > tol ? dd : (m > 0 ? tol : -tol);
        fb = refracted_angle(b, xoff, h, d, sq_eps);
    }
    *root = b;
    return true;
}

struct RowGeom {
    double rng, apt_m;
    int apt_smpl, apt_hsmpl;
};

// focus_rdrgrm's per-row scalars (simple_focusing.py:328-335).
__device__ RowGeom row_geom(const rp_focus_params& P, int64_t i, int64_t Nr) {
    RowGeom g;
    g.rng = __dadd_rn(__dmul_rn(P.rx_window_m, __ddiv_rn((double)i, (double)Nr)), P.rx_window_offset_m);
    g.apt_m = __dmul_rn(g.rng, P.sin_aperture);
    g.apt_smpl = (int)__ddiv_rn(__dmul_rn(2.0, g.apt_m), P.spacing);
    g.apt_hsmpl = (int)__ddiv_rn(g.apt_m, P.spacing);
    return g;
}

// Per (row, aperture sample): the source position (np.linspace), the
// straight slant range and its range bin (est_slant_range with clutter,
// slantrange_to_rangebin), and the matched-filter tap conj(exp(-4 pi i
// r / lam)) at the refraction-corrected range (get_target_phase).
__global__ void k_focus_geom(rp_focus_params P, int64_t Nr, int64_t row0, int nrows, int maxA, int* __restrict__ rb,
                             float2* __restrict__ mf, int* __restrict__ apt, int* __restrict__ err) {
    const int r = blockIdx.y;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    const int64_t i = row0 + r;
    const RowGeom g = row_geom(P, i, Nr);
    if (k == 0) {
        apt[2 * r] = g.apt_smpl;
        apt[2 * r + 1] = g.apt_hsmpl;
    }
    if (k >= g.apt_smpl || k >= maxA) return;
    // np.linspace(-apt_m, apt_m, apt_smpl): k * step + start, the last exactly stop
    const double start = -g.apt_m, stop = g.apt_m;
    double sx;
    if (g.apt_smpl > 1) {
        const double step = __ddiv_rn(__dsub_rn(stop, start), (double)(g.apt_smpl - 1));
        sx = (k == g.apt_smpl - 1) ? stop : __dadd_rn(__dmul_rn((double)k, step), start);
    } else {
        sx = start;
    }
    const double sz = P.altitude, tz = __dsub_rn(P.altitude, g.rng);
    const double dz = __dsub_rn(sz, tz);
    const double sl = __dsqrt_rn(__dadd_rn(__dmul_rn(sx, sx), __dmul_rn(dz, dz)));
    const double dm = __ddiv_rn(P.c1, P.rx_sample_rate);
    const double b = np_floor_divide(__dsub_rn(sl, P.rx_window_offset_m), dm);
    rb[(size_t)r * maxA + k] = (int)b;
    // matched filter: refraction angle on [0, 20 deg], then the two-way phase
    double th_r = 0.0;
    const double sq = sqrt(P.eps_2);
    if (!brent(fabs(sx), sz, tz, sq, 0.0, P.bracket_hi, &th_r)) {
        atomicMax(err, (int)(i + 1));
        th_r = 0.0;
    }
    const double th_i = asin(sq * sin(th_r));
    const double crng = sz / cos(th_i) + tz / cos(th_r) * sq;
    // phase 4 pi crng / lam, reduced in turns before the FP64 sine/cosine
    const double t = 2.0 * crng / P.lam;
    const double fr = t - rint(t);
    double s, c;
    sincospi(2.0 * fr, &s, &c);
    mf[(size_t)r * maxA + k] = make_float2((float)c, (float)s);      // conj(exp(-i phase))
}

template <class TI>
__device__ __forceinline__ float2 ld_c(const TI* p, size_t i);
template <>
__device__ __forceinline__ float2 ld_c<float2>(const float2* p, size_t i) { return __ldg(p + i); }
template <>
__device__ __forceinline__ float2 ld_c<double2>(const double2* p, size_t i) {
    const double2 v = __ldg(p + i);
    return make_float2((float)v.x, (float)v.y);
}
template <class TO>
__device__ __forceinline__ void st_c(TO* p, size_t i, float re, float im);
template <>
__device__ __forceinline__ void st_c<float2>(float2* p, size_t i, float re, float im) { p[i] = make_float2(re, im); }
template <>
__device__ __forceinline__ void st_c<double2>(double2* p, size_t i, float re, float im) {
    p[i] = make_double2(re, im);
}

// One pixel of focus_rdrgrm (simple_focusing.py:353-398): the window
// [a0, a1) of traces around j; row i of each column rolled by
// sltrng_rb[k] - i is element sltrng_rb[k] mod Nr; the kept FFT sample is
// sum_k row[k] mf[(n0 - k) mod L], L = 2 apt_smpl, n0 = (j - a0) + (L - w) / 2,
// with mf zero beyond apt_smpl.  Rows outside [row0, row0 + nrows) are zero.
template <class TI, class TO>
__global__ void k_focus_pix(const TI* __restrict__ rdr, int64_t Nr, int64_t Na, int64_t row0, int nrows, int maxA,
                            const int* __restrict__ rb, const float2* __restrict__ mf,
                            const int* __restrict__ apt, TO* __restrict__ out) {
    const int64_t i = blockIdx.y;
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= Na) return;
    const int64_t r = i - row0;
    if (r < 0 || r >= nrows) {
        st_c<TO>(out, (size_t)i * Na + j, 0.f, 0.f);
        return;
    }
    const int A = min(apt[2 * r], maxA), H = apt[2 * r + 1];
    const int64_t a0 = max((int64_t)0, j - H), a1 = min(Na, j + H);
    const int w = (int)(a1 - a0);
    const int L = 2 * A;
    const int n0 = (int)(j - a0) + (L - w) / 2;
    const int* rbr = rb + (size_t)r * maxA;
    const float2* mfr = mf + (size_t)r * maxA;
    float re0 = 0.f, im0 = 0.f, re1 = 0.f, im1 = 0.f;
    for (int k = 0; k < w; ++k) {
        int m = (n0 - k) % L;
        if (m < 0) m += L;
        if (m >= A) continue;
        int row = rbr[k] % (int)Nr;
        if (row < 0) row += (int)Nr;
        const float2 x = ld_c<TI>(rdr, (size_t)row * Na + a0 + k);
        const float2 f = __ldg(mfr + m);
        if (k & 1) {
            re1 = fmaf(x.x, f.x, fmaf(-x.y, f.y, re1));
            im1 = fmaf(x.x, f.y, fmaf(x.y, f.x, im1));
        } else {
            re0 = fmaf(x.x, f.x, fmaf(-x.y, f.y, re0));
            im0 = fmaf(x.x, f.y, fmaf(x.y, f.x, im0));
        }
    }
    st_c<TO>(out, (size_t)i * Na + j, re0 + re1, im0 + im1);
}

// full_focus_at_center (simple_focusing.py:137-183): rolled[r, k] =
// rdr[(r + shift_k) mod Nr, k]; out[r, j] = sum_k rolled[r, k] mf[j + Na/2 - k]
// over the taps 0 <= j + Na/2 - k < Na (the crop of the length-2Na circular
// convolution).  One block per (row, 256 outputs); taps staged in shared memory.
template <class TI, class TO>
__global__ void k_focus_center(const TI* __restrict__ rdr, int64_t Nr, int64_t Na, const int64_t* __restrict__ shift,
                               const float2* __restrict__ mf, TO* __restrict__ out) {
    __shared__ float2 s_row[256];
    __shared__ float2 s_mf[512];
    const int64_t r = blockIdx.y;
    const int64_t j0 = (int64_t)blockIdx.x * 256;
    const int64_t j = j0 + threadIdx.x;
    const int64_t h0 = Na / 2;
    float re0 = 0.f, im0 = 0.f, re1 = 0.f, im1 = 0.f;
    for (int64_t k0 = 0; k0 < Na; k0 += 256) {
        __syncthreads();
        {
            const int64_t k = k0 + threadIdx.x;
            float2 v = make_float2(0.f, 0.f);
            if (k < Na) {
                int64_t row = (r + shift[k]) % Nr;
                if (row < 0) row += Nr;
                v = ld_c<TI>(rdr, (size_t)row * Na + k);
            }
            s_row[threadIdx.x] = v;
            // taps m = j + h0 - k for j in the block and k in the tile:
            // m in [j0 + h0 - k0 - 255, j0 + h0 - k0 + 255]
            for (int t = threadIdx.x; t < 512; t += 256) {
                const int64_t m = j0 + h0 - k0 - 255 + t;
                s_mf[t] = (m >= 0 && m < Na) ? __ldg(mf + m) : make_float2(0.f, 0.f);
            }
        }
        __syncthreads();
        if (j < Na) {
            const int64_t kn = min((int64_t)256, Na - k0);
            for (int kk = 0; kk < kn; ++kk) {
                const float2 x = s_row[kk];
                const float2 f = s_mf[(int)(j - j0) + 255 - kk];
                if (kk & 1) {
                    re1 = fmaf(x.x, f.x, fmaf(-x.y, f.y, re1));
                    im1 = fmaf(x.x, f.y, fmaf(x.y, f.x, im1));
                } else {
                    re0 = fmaf(x.x, f.x, fmaf(-x.y, f.y, re0));
                    im0 = fmaf(x.x, f.y, fmaf(x.y, f.x, im0));
                }
            }
        }
    }
    if (j < Na) st_c<TO>(out, (size_t)r * Na + j, re0 + re1, im0 + im1);
}

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
};

int dmalloc(DevBuf& b, size_t bytes) {
    if (cudaMalloc(&b.p, std::max<size_t>(bytes, 16)) != cudaSuccess) {
        cudaGetLastError();
        rp_set_error("focusing: cudaMalloc of %zu bytes failed", bytes);
        return RP_ERR_NOMEM;
    }
    return RP_OK;
}

// The host's copy of row_geom for sizing (the device recomputes it exactly).
int host_max_aperture(const rp_focus_params& P, int64_t Nr, int64_t row0, int64_t nrows) {
    int m = 0;
    for (int64_t i = row0; i < row0 + nrows; ++i) {
        const double rng = P.rx_window_m * ((double)i / (double)Nr) + P.rx_window_offset_m;
        m = std::max(m, (int)(2.0 * (rng * P.sin_aperture) / P.spacing) + 1);
    }
    return m;
}

int check_params(const rp_focus_params* P) {
    if (!P || !(P->spacing > 0) || !(P->rx_sample_rate > 0) || !(P->lam > 0) || !(P->c1 > 0) ||
        !(P->eps_2 > 0) || !(P->bracket_hi > 0)) {
        rp_set_error("focusing: bad parameters (spacing, rx_sample_rate, lam, c1, eps_2 and the bracket must be > 0)");
        return RP_ERR_ARG;
    }
    return RP_OK;
}

}  // namespace

// Per-row geometry of focus_rdrgrm for rows [row0, row0 + nrows): apt_smpl
// and apt_hsmpl per row (apt, 2 ints per row), the range bins (rb) and the
// matched filter (mf, complex64 as 2 floats) of each aperture sample, rows
// of stride maxA.  Host buffers.
extern "C" int rp_focus_geometry(const rp_focus_params* P, int64_t Nr, int64_t row0, int64_t nrows, int maxA,
                                 int* apt, int* rb, float* mf) {
    int rc = check_params(P);
    if (rc) return rc;
    if (Nr <= 0 || row0 < 0 || nrows <= 0 || row0 + nrows > Nr || maxA <= 0 || !apt || !rb || !mf) {
        rp_set_error("rp_focus_geometry: bad argument");
        return RP_ERR_ARG;
    }
    DevBuf d_rb, d_mf, d_apt, d_err;
    if ((rc = dmalloc(d_rb, sizeof(int) * nrows * maxA)) || (rc = dmalloc(d_mf, sizeof(float2) * nrows * maxA)) ||
        (rc = dmalloc(d_apt, sizeof(int) * 2 * nrows)) || (rc = dmalloc(d_err, sizeof(int))))
        return rc;
    RP_CUDA(cudaMemset(d_err.p, 0, sizeof(int)));
    RP_CUDA(cudaMemset(d_rb.p, 0, sizeof(int) * nrows * maxA));
    RP_CUDA(cudaMemset(d_mf.p, 0, sizeof(float2) * nrows * maxA));
    k_focus_geom<<<dim3((maxA + 127) / 128, (unsigned)nrows), 128>>>(*P, Nr, row0, (int)nrows, maxA, (int*)d_rb.p,
                                                                   (float2*)d_mf.p, (int*)d_apt.p, (int*)d_err.p);
    RP_CUDA(cudaGetLastError());
    int err = 0;
    RP_CUDA(cudaMemcpy(&err, d_err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {
        rp_set_error("focusing: no refraction angle in [0, bracket] for range row %d", err - 1);
        return RP_ERR_ARG;
    }
    RP_CUDA(cudaMemcpy(apt, d_apt.p, sizeof(int) * 2 * nrows, cudaMemcpyDeviceToHost));
    RP_CUDA(cudaMemcpy(rb, d_rb.p, sizeof(int) * nrows * maxA, cudaMemcpyDeviceToHost));
    RP_CUDA(cudaMemcpy(mf, d_mf.p, sizeof(float2) * nrows * maxA, cudaMemcpyDeviceToHost));
    return RP_OK;
}

extern "C" int rp_focus_aperture(const rp_focus_params* P, const void* rdr, int64_t Nr, int64_t Na, int in128,
                                 int64_t row_lo, int64_t row_hi, void* out, int out128, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    int rc = check_params(P);
    if (rc) return rc;
    if (!rdr || !out || Nr <= 0 || Na <= 0 || Nr > INT32_MAX || row_lo < 0 || row_hi >= Nr || row_lo > row_hi) {
        rp_set_error("rp_focus_aperture: bad argument (rows [%lld, %lld] of %lld)", (long long)row_lo,
                     (long long)row_hi, (long long)Nr);
        return RP_ERR_ARG;
    }
    const int64_t nrows = row_hi - row_lo + 1;
    const int maxA = host_max_aperture(*P, Nr, row_lo, nrows);
    const size_t ein = in128 ? 16 : 8, eout = out128 ? 16 : 8;
    DevBuf d_in, d_out, d_rb, d_mf, d_apt, d_err;
    if ((rc = dmalloc(d_in, ein * Nr * Na)) || (rc = dmalloc(d_out, eout * Nr * Na)) ||
        (rc = dmalloc(d_rb, sizeof(int) * nrows * maxA)) || (rc = dmalloc(d_mf, sizeof(float2) * nrows * maxA)) ||
        (rc = dmalloc(d_apt, sizeof(int) * 2 * nrows)) || (rc = dmalloc(d_err, sizeof(int))))
        return rc;
    RP_CUDA(cudaMemcpyAsync(d_in.p, rdr, ein * Nr * Na, cudaMemcpyHostToDevice, st));
    RP_CUDA(cudaMemsetAsync(d_err.p, 0, sizeof(int), st));
    k_focus_geom<<<dim3((maxA + 127) / 128, (unsigned)nrows), 128, 0, st>>>(
        *P, Nr, row_lo, (int)nrows, maxA, (int*)d_rb.p, (float2*)d_mf.p, (int*)d_apt.p, (int*)d_err.p);
    RP_LAUNCHED();
    const dim3 grid((unsigned)((Na + 255) / 256), (unsigned)Nr);
#define RP_PIX(TI, TO) k_focus_pix<TI, TO><<<grid, 256, 0, st>>>((const TI*)d_in.p, Nr, Na, row_lo, (int)nrows, maxA, \
        (const int*)d_rb.p, (const float2*)d_mf.p, (const int*)d_apt.p, (TO*)d_out.p)
    if (in128 && out128) RP_PIX(double2, double2);
    else if (in128) RP_PIX(double2, float2);
    else if (out128) RP_PIX(float2, double2);
    else RP_PIX(float2, float2);
#undef RP_PIX
    RP_LAUNCHED();
    int err = 0;
    RP_CUDA(cudaMemcpyAsync(&err, d_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    RP_CUDA(cudaMemcpyAsync(out, d_out.p, eout * Nr * Na, cudaMemcpyDeviceToHost, st));
    RP_CUDA(cudaStreamSynchronize(st));
    if (err) {
        rp_set_error("focusing: no refraction angle in [0, bracket] for range row %d", err - 1);
        return RP_ERR_ARG;
    }
    return RP_OK;
}

extern "C" int rp_focus_center(const void* rdr, int64_t Nr, int64_t Na, int in128, const int64_t* shifts,
                               const float* mf, void* out, int out128, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (!rdr || !out || !shifts || !mf || Nr <= 0 || Na <= 0) {
        rp_set_error("rp_focus_center: bad argument");
        return RP_ERR_ARG;
    }
    const size_t ein = in128 ? 16 : 8, eout = out128 ? 16 : 8;
    DevBuf d_in, d_out, d_sh, d_mf;
    int rc;
    if ((rc = dmalloc(d_in, ein * Nr * Na)) || (rc = dmalloc(d_out, eout * Nr * Na)) ||
        (rc = dmalloc(d_sh, sizeof(int64_t) * Na)) || (rc = dmalloc(d_mf, sizeof(float2) * Na)))
        return rc;
    RP_CUDA(cudaMemcpyAsync(d_in.p, rdr, ein * Nr * Na, cudaMemcpyHostToDevice, st));
    RP_CUDA(cudaMemcpyAsync(d_sh.p, shifts, sizeof(int64_t) * Na, cudaMemcpyHostToDevice, st));
    RP_CUDA(cudaMemcpyAsync(d_mf.p, mf, sizeof(float2) * Na, cudaMemcpyHostToDevice, st));
    const dim3 grid((unsigned)((Na + 255) / 256), (unsigned)Nr);
#define RP_CEN(TI, TO) k_focus_center<TI, TO><<<grid, 256, 0, st>>>((const TI*)d_in.p, Nr, Na, \
        (const int64_t*)d_sh.p, (const float2*)d_mf.p, (TO*)d_out.p)
    if (in128 && out128) RP_CEN(double2, double2);
    else if (in128) RP_CEN(double2, float2);
    else if (out128) RP_CEN(float2, double2);
    else RP_CEN(float2, float2);
#undef RP_CEN
    RP_LAUNCHED();
    RP_CUDA(cudaMemcpyAsync(out, d_out.p, eout * Nr * Na, cudaMemcpyDeviceToHost, st));
    RP_CUDA(cudaStreamSynchronize(st));
    return RP_OK;
}
