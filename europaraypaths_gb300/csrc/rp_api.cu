// rp_api.cu -- C ABI of libraypath: errors, parameters, resident scenes,
// spectral tables, and the rp_simulate dispatch to the two forms.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <utility>
#include <vector>

#include "rp_internal.h"
#include "rp_fft.cuh"

// ---------------------------------------------------------------- errors --
static thread_local char g_err[1024] = "";
thread_local int64_t g_launches = 0;
thread_local StageTimer g_timer;

void StageTimer::mark(int i, cudaStream_t st) {
    if (!enabled) return;
    if (!have_events) {
        for (int k = 0; k <= RP_NSTAGE; ++k) cudaEventCreate(&ev[k]);
        have_events = 1;
    }
    cudaEventRecord(ev[i], st);
}

void StageTimer::collect(int first, int last) {
    if (!enabled || !have_events) return;
    for (int k = first; k < last; ++k) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, ev[k], ev[k + 1]) == cudaSuccess) ms[k] += t;
    }
}

void rp_set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int rp_cuda_fail(cudaError_t e, const char* what) {
    rp_set_error("CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
    return RP_ERR_CUDA;
}

// Kernels whose dynamic shared memory depends on the scene are launched
// from several host threads (server workers).  Their limit only ever grows,
// per device and under a lock, so no launch meets a limit that another
// thread lowered between this thread's raise and its launch.
int rp_allow_dyn_smem(const void* fn, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> cur;
    // the 48 KiB allowed without the attribute covers static and dynamic
    // shared memory together, so any dynamic size sets it
    if (bytes == 0) return RP_OK;
    int dev = 0;
    RP_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    size_t& c = cur[{dev, fn}];
    if (bytes <= c) return RP_OK;
    RP_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    c = bytes;
    return RP_OK;
}

int Arena::reserve(size_t bytes) {
    if (bytes <= cap) return RP_OK;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 8 + (1 << 20);
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        rp_set_error("device scratch allocation of %zu bytes failed: %s", want, cudaGetErrorString(e));
        return RP_ERR_NOMEM;
    }
    cap = want;
    return RP_OK;
}

void Arena::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    off = 0;
}

extern "C" const char* rp_version(void) { return "raypath-gb300 1.0 (sm_103a)"; }

extern "C" int rp_last_error(char* buf, size_t len) {
    if (!buf || len == 0) return RP_ERR_ARG;
    snprintf(buf, len, "%s", g_err);
    return RP_OK;
}

extern "C" int rp_set_timing(int enable) {
    g_timer.enabled = enable ? 1 : 0;
    return RP_OK;
}

extern "C" int rp_last_timing(double* ms, int n) {
    if (!ms || n < 0) return RP_ERR_ARG;
    for (int i = 0; i < n && i < RP_NSTAGE; ++i) ms[i] = g_timer.ms[i];
    if (n > RP_NSTAGE) ms[RP_NSTAGE] = (double)g_timer.pair_launches;
    return RP_OK;
}

extern "C" int rp_last_launch_count(int64_t* n) {
    if (!n) return RP_ERR_ARG;
    *n = g_launches;
    return RP_OK;
}

// ------------------------------------------------------------ parameters --
// Derivations of parseSimulationParameters, src/CUDA/file_io.cu:167-213.
extern "C" int rp_params_derive(rp_params* p) {
    if (!p) { rp_set_error("rp_params_derive: null params"); return RP_ERR_ARG; }
    if (!(p->frequency > 0) || !(p->bandwidth > 0) || !(p->rx_sample_rate > 0) ||
        !(p->rx_window_m > 0) || !(p->eps_1 > 0) || !(p->eps_2 > 0) || !(p->fs > 0)) {
        rp_set_error("rp_params_derive: frequency, bandwidth, rx_sample_rate, rx_window_m, "
                     "eps_1, eps_2 and fs must be positive");
        return RP_ERR_ARG;
    }
    const double c = 299792458.0;
    p->c = c;
    p->rng_res = c / p->bandwidth;
    p->lam = c / p->frequency;
    p->k = 2 * RP_PI_F / p->lam;
    p->grefr_lin = std::pow(10.0, p->subsurface_gain / 10.0);
    p->grefl_lin = std::pow(10.0, p->surface_gain / 10.0);
    p->ks = p->k * p->rms_height;
    p->c_1 = c / std::sqrt(p->eps_1);
    p->c_2 = c / std::sqrt(p->eps_2);
    p->nu_1 = 376.7 / std::sqrt(p->eps_1);
    p->nu_2 = 376.7 / std::sqrt(p->eps_2);
    auto alpha = [&](double sig, double eps) {
        double epp = sig / (2 * RP_PI_FRIIS * p->frequency * 8.85e-12);
        double a = std::sqrt(1 + (epp / eps) * (epp / eps)) - 1;
        a = std::sqrt(0.5 * eps * a);
        return (a * 2 * RP_PI_FRIIS) / p->lam;
    };
    p->alpha1 = alpha(p->sig_1, p->eps_1);
    p->alpha2 = alpha(p->sig_2, p->eps_2);
    // nr keeps the reference's float expression (file_io.cu:212) bit for bit.
    float nrf = ((float)p->rx_window_m / 299792480.0f) * (float)p->rx_sample_rate;
    if (!(nrf >= 2.0f) || nrf > 1.0e6f) {
        rp_set_error("rp_params_derive: rx_window_m and rx_sample_rate give %g range bins", (double)nrf);
        return RP_ERR_ARG;
    }
    p->nr = (int32_t)nrf;
    p->dr = p->rx_window_m / (double)p->nr;
    return RP_OK;
}

// loadAttenPrismFile's conductivity -> alpha, src/CUDA/file_io.cu:501-505.
extern "C" int rp_prism_alpha(const rp_params* p, double sig, double* alpha) {
    if (!p || !alpha) { rp_set_error("rp_prism_alpha: null argument"); return RP_ERR_ARG; }
    double epp = sig / (2 * RP_PI_FRIIS * p->frequency * 8.85e-12);
    double a = std::sqrt(1 + (epp / p->eps_2) * (epp / p->eps_2)) - 1;
    a = std::sqrt(0.5 * p->eps_2 * a);
    *alpha = (a * 2 * RP_PI_FRIIS) / p->lam;
    return RP_OK;
}

// ----------------------------------------------------------- host tables --
using cd = std::complex<double>;

static void host_fft(std::vector<cd>& a, int sign) {
    const int n = (int)a.size();
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(a[i], a[j]);
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1;
        for (int k = 0; k < half; ++k) {
            double ang = sign * 2.0 * RP_PI * k / len;
            cd w(std::cos(ang), std::sin(ang));
            for (int i = 0; i < n; i += len) {
                cd u = a[i + k], v = a[i + k + half] * w;
                a[i + k] = u + v;
                a[i + k + half] = u - v;
            }
        }
    }
}

static double host_sinc(double x) {
    if (std::fabs(x) < 1e-6) return 1.0;
    return std::sin(RP_PI * x) / (RP_PI * x);
}

template <class T>
static int upload(T** dst, const void* src, size_t bytes, size_t* acc) {
    if (bytes == 0) { *dst = nullptr; return RP_OK; }
    RP_CUDA(cudaMalloc((void**)dst, bytes));
    RP_CUDA(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
    if (acc) *acc += bytes;
    return RP_OK;
}

static int upload_cplx(const std::vector<cd>& v, double** d64, float** d32, size_t* acc) {
    std::vector<double> a(2 * v.size());
    std::vector<float> b(2 * v.size());
    for (size_t i = 0; i < v.size(); ++i) {
        a[2 * i] = v[i].real(); a[2 * i + 1] = v[i].imag();
        b[2 * i] = (float)v[i].real(); b[2 * i + 1] = (float)v[i].imag();
    }
    int rc = upload(d64, a.data(), a.size() * sizeof(double), acc);
    if (rc) return rc;
    return upload(d32, b.data(), b.size() * sizeof(float), acc);
}

static std::vector<cd> twiddles(int n) {
    std::vector<cd> t(n / 2);
    for (int k = 0; k < n / 2; ++k) {
        double ang = -2.0 * RP_PI * k / n;
        t[k] = cd(std::cos(ang), std::sin(ang));
    }
    return t;
}

static bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// Bluestein chirp w_k = e^{-i pi k^2 / n} (angle reduced exactly mod 2 pi).
static std::vector<cd> bluestein_chirp(int n) {
    std::vector<cd> w(n);
    for (int k = 0; k < n; ++k) {
        long long kk = ((long long)k * k) % (2LL * n);
        double ang = -RP_PI * (double)kk / n;
        w[k] = cd(std::cos(ang), std::sin(ang));
    }
    return w;
}

static std::vector<cd> bluestein_kernel(const std::vector<cd>& w, int M) {
    const int n = (int)w.size();
    std::vector<cd> b(M, cd(0, 0));
    for (int k = 0; k < n; ++k) {
        b[k] = std::conj(w[k]);
        if (k) b[M - k] = std::conj(w[k]);
    }
    host_fft(b, -1);
    return b;
}

// Forward DFT of any length on the host (FP64), cuFFT sign convention.
static std::vector<cd> host_dft(std::vector<cd> x) {
    const int n = (int)x.size();
    if (is_pow2(n)) { host_fft(x, -1); return x; }
    int M = 1;
    while (M < 2 * n - 1) M <<= 1;
    std::vector<cd> w = bluestein_chirp(n), b = bluestein_kernel(w, M), y(M, cd(0, 0));
    for (int k = 0; k < n; ++k) y[k] = x[k] * w[k];
    host_fft(y, -1);
    for (int k = 0; k < M; ++k) y[k] *= b[k];
    host_fft(y, +1);
    for (int k = 0; k < n; ++k) x[k] = y[k] * w[k] / (double)M;
    return x;
}

static int build_plan(DftPlan& pl, int n, size_t* acc) {
    pl.n = n;
    pl.pow2 = is_pow2(n);
    int M = 1;
    if (pl.pow2) M = n;
    else while (M < 2 * n - 1) M <<= 1;
    int l = 0;
    while ((1 << l) < M) ++l;
    pl.log2M = l;
    int rc = upload_cplx(twiddles(M), &pl.tw64, &pl.tw32, acc);
    if (rc || pl.pow2) return rc;
    std::vector<cd> w = bluestein_chirp(n);
    if ((rc = upload_cplx(w, &pl.bw64, &pl.bw32, acc))) return rc;
    return upload_cplx(bluestein_kernel(w, M), &pl.bW64, &pl.bW32, acc);
}

static void free_plan(DftPlan& pl) {
    void* ptrs[] = {pl.tw64, pl.bw64, pl.bW64, pl.tw32, pl.bw32, pl.bW32};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    pl = DftPlan();
}

static int build_tables(rp_scene* s) {
    const rp_params& p = s->p;
    const int nr = p.nr;
    s->nr = nr;
    size_t acc = 0;
    int rc;
    if ((rc = build_plan(s->plan2, 2 * nr, &acc))) return rc;
    if ((rc = build_plan(s->planN, 2 * nr - 1, &acc))) return rc;
    // chirp spectra (genCenteredChirpPadded, radar_kernels.cu:489-503)
    std::vector<cd> c1(2 * nr), c2(2 * nr);
    for (int i = 0; i < 2 * nr; ++i) {
        double off = (double)(i - nr / 2) * p.dr;
        c1[i] = cd(host_sinc(off / p.rng_res), 0.0);
        c2[i] = cd(host_sinc(off / (2 * p.rng_res)), 0.0);
    }
    if ((rc = upload_cplx(host_dft(c1), &s->d_C1_64, &s->d_C1_32, &acc))) return rc;
    if ((rc = upload_cplx(host_dft(c2), &s->d_C2_64, &s->d_C2_32, &acc))) return rc;
    if (s->dp.cmode == 1) {
        // genChirp (radar_kernels.cu:454-466): sinc(i dr / res) + its wrap at nr
        if ((rc = build_plan(s->planR, nr, &acc))) return rc;
        std::vector<cd> cr(nr);
        for (int i = 0; i < nr; ++i)
            cr[i] = cd(host_sinc((double)i * p.dr / p.rng_res) + host_sinc((double)(i - nr) * p.dr / p.rng_res), 0.0);
        if ((rc = upload_cplx(host_dft(cr), &s->d_CR_64, &s->d_CR_32, &acc))) return rc;
    }
    // cropSpectrum (elementary_kernels.cu:258-278): keep |freq_k| <= B on the
    // N-point grid; the kept set is min(k, N-k) <= K.
    const int N = 2 * nr - 1;
    int K = -1;
    for (int m = 0; m <= N / 2; ++m)
        if (!(std::fabs((double)m * p.rx_sample_rate / N) > p.bandwidth)) K = m;
    s->crop_K = K;
    s->crop_all = (K >= N / 2);
    // shared-memory path tables: nr a power of two (>= 16: the compression
    // kernel's outer passes hold 16 elements a thread), M = 4 nr
    if (is_pow2(nr) && nr >= 16) {
        const int n2 = 2 * nr, M = 4 * nr;
        int lM = 0;
        while ((1 << lM) < M) ++lM;
        std::vector<Cplx<double>> tw(M);
        for (int k = 0; k < M; ++k) {
            double ang = -2.0 * RP_PI * k / M;
            tw[k] = Cplx<double>{std::cos(ang), std::sin(ang)};
        }
        struct TWH {
            const std::vector<Cplx<double>>* t;
            Cplx<double> operator()(int k) const { return (*t)[k]; }
        } f{&tw};
        auto to32 = [](const std::vector<Cplx<double>>& v, float** d, size_t* a) {
            std::vector<float> b(2 * v.size());
            for (size_t i = 0; i < v.size(); ++i) { b[2 * i] = (float)v[i].x; b[2 * i + 1] = (float)v[i].y; }
            return upload(d, b.data(), b.size() * sizeof(float), a);
        };
        // the targets' chirp: genCenteredChirpPadded(2 rng_res), or the surface
        // chirp (rng_res) in specular mode, which never regenerates it
        // (sim.cu:851-856)
        const double tres = s->dp.specular ? p.rng_res : 2 * p.rng_res;
        std::vector<Cplx<double>> c2(n2), h(M, Cplx<double>{0, 0});
        for (int i = 0; i < n2; ++i) c2[i] = Cplx<double>{host_sinc((double)(i - nr / 2) * p.dr / tres), 0.0};
        if (n2 == 2 * RP_CONV_CHUNK) {
            // the compression runs these transforms by halves: DIF_n's first
            // (span-n radix-2) stage, then DIF of each half of length nr
            for (int e = 0; e < nr; ++e) {
                const Cplx<double> a = c2[e], b = c2[e + nr];
                const Cplx<double> d{a.x - b.x, a.y - b.y};
                const double ang = -2.0 * RP_PI * e / n2;
                const double cw = std::cos(ang), sw = std::sin(ang);
                c2[e] = Cplx<double>{a.x + b.x, a.y + b.y};
                c2[e + nr] = Cplx<double>{d.x * cw - d.y * sw, d.x * sw + d.y * cw};
            }
            host_dif(c2.data(), nr, f, lM);
            host_dif(c2.data() + nr, nr, f, lM);
        } else {
            host_dif(c2.data(), n2, f, lM);
        }
        // cropSpectrum followed by the inverse N-point DFT is a circular
        // convolution with h[n] = (1/N) sum_{min(k,N-k) <= K} e^{2 pi i k n / N}
        // = sin(pi (2K+1) n / N) / (N sin(pi n / N)) (the Dirichlet kernel of
        // the kept band; a delta when nothing is cropped).  Its M-point
        // spectrum, with the 1/M of the unnormalised inverse, in DIF order.
        for (int n = 0; n < N; ++n) {
            double v;
            if (s->crop_all) v = (n == 0) ? 1.0 : 0.0;
            else if (n == 0) v = (double)(2 * K + 1) / N;
            else {
                const long long r = ((long long)(2 * K + 1) * n) % (2LL * N);
                v = std::sin(RP_PI * (double)r / N) / ((double)N * std::sin(RP_PI * (double)n / N));
            }
            h[n] = Cplx<double>{v / M, 0.0};
        }
        host_dif(h.data(), M, f, lM);
        if ((rc = to32(c2, &s->d_C2S, &acc))) return rc;
        if ((rc = to32(h, &s->d_HS, &acc))) return rc;
        s->mS = M;
        s->log2mS = lM;
        s->smem_conv = 1;
    }
    s->store_bytes += acc;
    return RP_OK;
}

// Whether every facet's frame (n, u, v) is orthonormal to 1e-5 (unit
// lengths, pairwise dot products): the fast form then forms the incidence
// angle from the tangent components alone.  The generators that build u and
// v by cross products give such frames; frames with independently
// normalised slope tangents do not.
static int frames_orthonormal(const double* F, int64_t nf) {
    const double tol = 1e-5;
    for (int64_t i = 0; i < nf; ++i) {
        const double n[3] = {F[3 * nf + i], F[4 * nf + i], F[5 * nf + i]};
        const double u[3] = {F[6 * nf + i], F[7 * nf + i], F[8 * nf + i]};
        const double v[3] = {F[9 * nf + i], F[10 * nf + i], F[11 * nf + i]};
        auto dot = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
        if (!(std::fabs(dot(n, n) - 1.0) <= tol && std::fabs(dot(u, u) - 1.0) <= tol &&
              std::fabs(dot(v, v) - 1.0) <= tol && std::fabs(dot(n, u)) <= tol && std::fabs(dot(n, v)) <= tol &&
              std::fabs(dot(u, v)) <= tol))
            return 0;
    }
    return 1;
}

// Bounding spheres (centre, radius) of every RP_CULL_TILE consecutive facets
// of a [12][nf] FP64 store, for the culling kernel's tile test.  The radius
// is inflated far beyond FP64 rounding so the test stays conservative.
static std::vector<double> tile_spheres(const double* F, int64_t nf) {
    const int64_t nt = (nf + RP_CULL_TILE - 1) / RP_CULL_TILE;
    std::vector<double> out((size_t)4 * nt);
    for (int64_t t = 0; t < nt; ++t) {
        const int64_t i0 = t * RP_CULL_TILE, i1 = std::min(nf, i0 + RP_CULL_TILE);
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int64_t i = i0; i < i1; ++i)
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], F[a * nf + i]);
                hi[a] = std::max(hi[a], F[a * nf + i]);
            }
        const double c[3] = {0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1]), 0.5 * (lo[2] + hi[2])};
        double r2 = 0.0;
        for (int64_t i = i0; i < i1; ++i) {
            double q = 0.0;
            for (int a = 0; a < 3; ++a) q += (F[a * nf + i] - c[a]) * (F[a * nf + i] - c[a]);
            r2 = std::max(r2, q);
        }
        const double cn = std::fabs(c[0]) + std::fabs(c[1]) + std::fabs(c[2]);
        out[4 * t] = c[0]; out[4 * t + 1] = c[1]; out[4 * t + 2] = c[2];
        out[4 * t + 3] = std::sqrt(r2) * (1.0 + 1e-9) + 1e-9 * (1.0 + cn);
    }
    return out;
}

// Morton order of facet centres (spatial locality for the fast form).
static uint64_t spread16(uint32_t v) {
    uint64_t x = v & 0xffff;
    x = (x | (x << 8)) & 0x00ff00ff;
    x = (x | (x << 4)) & 0x0f0f0f0f;
    x = (x | (x << 2)) & 0x33333333;
    x = (x | (x << 1)) & 0x55555555;
    return x;
}

extern "C" int rp_scene_create(const rp_params* p, const double* facets, int64_t nf,
                               const double* targets, int64_t nt, const double* prisms,
                               int64_t np, int device, rp_scene** out) {
    if (!p || !out || nf < 0 || nt < 0 || np < 0 || (nf > 0 && !facets) ||
        (nt > 0 && !targets) || (np > 0 && !prisms)) {
        rp_set_error("rp_scene_create: bad argument");
        return RP_ERR_ARG;
    }
    if (nf > (int64_t)1 << 31) { rp_set_error("rp_scene_create: more than 2^31 facets"); return RP_ERR_ARG; }
    if (p->nr <= 0 || !(p->lam > 0)) {
        rp_set_error("rp_scene_create: parameters not derived (call rp_params_derive)");
        return RP_ERR_ARG;
    }
    // Modes (sim.cu:733-986).  The reference defines: the default
    // (non-specular, linear convolution); specular with linear convolution;
    // specular without convolution or with circular convolution for ttype-0
    // targets only.  Non-specular without linear convolution writes a 2nr
    // chirp into an nr (or unallocated) buffer (sim.cu:411-438, 851-856), and
    // ttype-1 targets without linear convolution use an unallocated chirp and
    // temp buffer (sim.cu:864-872, 912): refused.  incoherent mode takes its
    // surface phases from a seeded hash (rp_incoherent_turns) instead of
    // clock64().
    const bool lin = p->convolution && p->convolution_linear;
    if (!p->specular && !lin) {
        rp_set_error("rp_scene_create: non-specular mode needs convolution=true, convolution_linear=true");
        return RP_ERR_UNSUPPORTED;
    }
    if (p->specular && !lin)
        for (int64_t t = 0; t < nt; ++t)
            if (targets[6 * nt + t] != 0.0) {
                rp_set_error("rp_scene_create: specular mode without linear convolution supports ttype-0 "
                             "targets only");
                return RP_ERR_UNSUPPORTED;
            }
    *out = nullptr;
    RP_CUDA(cudaSetDevice(device));
    rp_scene* s = new rp_scene();
    s->p = *p;
    s->device = device;
    s->nf = nf; s->nt = nt; s->np = np;
    DevParams& d = s->dp;
    d.lam = p->lam; d.fs = p->fs; d.P = p->power; d.nidx = std::sqrt(p->eps_2);
    d.eps1 = p->eps_1; d.eps2 = p->eps_2; d.nu1 = p->nu_1; d.nu2 = p->nu_2;
    d.alpha1 = p->alpha1; d.alpha2 = p->alpha2; d.ks = p->ks; d.c1_over_c2 = p->c_1 / p->c_2;
    d.dr = p->dr; d.smpl = p->rx_sample_rate; d.B = p->bandwidth; d.rng_res = p->rng_res;
    d.ap_rad = p->aperture * (RP_PI / 180.0);
    d.ap_cos = std::cos(d.ap_rad);
    d.turn = RP_PI_F / (RP_PI * p->lam);
    d.inv_dr = 1.0 / p->dr;
    d.sqrt_eps12 = std::sqrt(p->eps_1 / p->eps_2);
    d.nr = p->nr; d.lossless = p->lossless; d.disable_surface = p->disable_surface;
    d.rerad_funct = p->rerad_funct;
    d.specular = p->specular ? 1 : 0;
    d.incoherent = p->incoherent ? 1 : 0;
    d.inc_seed = (unsigned long long)p->incoherent_seed;
    d.cmode = !p->convolution ? 2 : (p->convolution_linear ? 0 : 1);
    d.c_over_c2 = p->c / p->c_2;
    int rc;
    auto fail = [&](int code) { rp_scene_destroy(s); return code; };
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return fail(rp_cuda_fail(cudaGetLastError(), "cudaGetDeviceProperties"));
    s->sm_count = prop.multiProcessorCount;
    if ((rc = upload(&s->d_facets, facets, sizeof(double) * 12 * nf, &s->store_bytes))) return fail(rc);
    if ((rc = upload(&s->d_targets, targets, sizeof(double) * 7 * nt, &s->store_bytes))) return fail(rc);
    if ((rc = upload(&s->d_prisms, prisms, sizeof(double) * 7 * np, &s->store_bytes))) return fail(rc);
    if (nt > 0) s->h_targets.assign(targets, targets + 7 * nt);
    for (int64_t t = 0; t < nt; ++t)
        if (targets[6 * nt + t] == 0.0) { s->any_ttype0 = 1; break; }
    s->d_targets_fast = s->d_targets;
    s->nt1 = nt;
    if (s->any_ttype0) {
        std::vector<int64_t> perm;
        for (int pass = 0; pass < 2; ++pass)
            for (int64_t t = 0; t < nt; ++t)
                if ((targets[6 * nt + t] == 0.0) == (pass == 1)) perm.push_back(t);
        std::vector<double> tf((size_t)7 * nt);
        for (int c = 0; c < 7; ++c)
            for (int64_t i = 0; i < nt; ++i) tf[(size_t)c * nt + i] = targets[(size_t)c * nt + perm[i]];
        s->nt1 = 0;
        while (s->nt1 < nt && tf[(size_t)6 * nt + s->nt1] != 0.0) ++s->nt1;
        if ((rc = upload(&s->d_targets_fast, tf.data(), sizeof(double) * 7 * nt, &s->store_bytes))) return fail(rc);
    }
    // spatially sorted copy for the fast form
    if (nf > 0) {
        double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
        for (int64_t i = 0; i < nf; ++i) {
            xmin = std::min(xmin, facets[i]); xmax = std::max(xmax, facets[i]);
            ymin = std::min(ymin, facets[nf + i]); ymax = std::max(ymax, facets[nf + i]);
        }
        double sx = (xmax > xmin) ? 65535.0 / (xmax - xmin) : 0.0;
        double sy = (ymax > ymin) ? 65535.0 / (ymax - ymin) : 0.0;
        std::vector<uint64_t> key(nf);
        for (int64_t i = 0; i < nf; ++i) {
            uint32_t qx = (uint32_t)std::lround((facets[i] - xmin) * sx);
            uint32_t qy = (uint32_t)std::lround((facets[nf + i] - ymin) * sy);
            key[i] = (spread16(qy) << 1) | spread16(qx);
        }
        std::vector<int64_t> order(nf);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return key[a] < key[b]; });
        std::vector<double> sorted((size_t)12 * nf);
        for (int c = 0; c < 12; ++c)
            for (int64_t i = 0; i < nf; ++i) sorted[(size_t)c * nf + i] = facets[(size_t)c * nf + order[i]];
        if ((rc = upload(&s->d_order, order.data(), sizeof(int64_t) * nf, &s->store_bytes))) return fail(rc);
        if ((rc = upload(&s->d_sorted, sorted.data(), sizeof(double) * 12 * nf, &s->store_bytes))) return fail(rc);
        const std::vector<double> ts = tile_spheres(sorted.data(), nf), tf = tile_spheres(facets, nf);
        if ((rc = upload(&s->d_tiles_sorted, ts.data(), sizeof(double) * ts.size(), &s->store_bytes))) return fail(rc);
        s->h_tiles_sorted = ts;
        if ((rc = upload(&s->d_tiles_file, tf.data(), sizeof(double) * tf.size(), &s->store_bytes))) return fail(rc);
    }
    if ((rc = build_tables(s))) return fail(rc);
    // specular mode evaluates cos Tth from the normal: general-frame records
    s->ortho = (nf > 0 && !p->specular) ? frames_orthonormal(facets, nf) : 0;
    if (const char* v = getenv("RP_PAIR_ORTHO")) s->ortho = s->ortho && atoi(v) != 0;   // 0: general frames
    s->dp.ortho = s->ortho;
    if (const char* v = getenv("RP_PAIR_VARIANT")) s->pair_variant = atoi(v) == 1 ? 1 : 0;
    // 0-3 for one segment (taken & 3), 4-9 also for multi-segment waves
    if (const char* v = getenv("RP_PAIR_CFG")) s->pair_cfg = std::max(0, std::min(9, atoi(v)));
    // test mode of the timeout path: the pair kernels issue no bulk copy and
    // give up after a short bounded wait, so the call returns RP_ERR_TIMEOUT
    // with nothing in flight
    if (const char* v = getenv("RP_TEST_STALL_COPIES")) {
        if (atoi(v) != 0) { s->stall_copies = 1; s->spin_limit = RP_SPIN_LIMIT_TEST; }
    }
    cudaError_t e = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail(rp_cuda_fail(e, "cudaStreamCreate"));
    *out = s;
    return RP_OK;
}

extern "C" int rp_scene_destroy(rp_scene* s) {
    if (!s) return RP_OK;
    cudaSetDevice(s->device);
    if (s->own_stream) cudaStreamSynchronize(s->own_stream);
    if (s->d_targets_fast && s->d_targets_fast != s->d_targets) cudaFree(s->d_targets_fast);
    void* ptrs[] = {s->d_facets, s->d_targets, s->d_prisms, s->d_order, s->d_sorted, s->d_tiles_sorted, s->d_tiles_file,
                    s->d_C1_64, s->d_C2_64, s->d_C1_32, s->d_C2_32, s->d_C2S,
                    s->d_HS, s->d_CR_64, s->d_CR_32};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    free_plan(s->plan2);
    free_plan(s->planN);
    free_plan(s->planR);
    s->ws.arena.release();
    s->ws.arena2.release();
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
    delete s;
    return RP_OK;
}

extern "C" int rp_scene_footprint(const rp_scene* s, int64_t* bytes) {
    if (!s || !bytes) { rp_set_error("rp_scene_footprint: null argument"); return RP_ERR_ARG; }
    *bytes = (int64_t)s->store_bytes;
    return RP_OK;
}

extern "C" int rp_query_footprint(const rp_scene* s, int64_t ns, int form, int64_t* bytes) {
    if (!s || !bytes || ns < 0) { rp_set_error("rp_query_footprint: bad argument"); return RP_ERR_ARG; }
    int f = form & 0xff;
    if (f == RP_FORM_PLAIN_F64) *bytes = (int64_t)rp_plain_scratch(s, ns);
    else if (f == RP_FORM_FAST_F32) *bytes = (int64_t)rp_fast_scratch(s, ns);
    else { rp_set_error("rp_query_footprint: unknown form %d", form); return RP_ERR_ARG; }
    return RP_OK;
}

static int run_form(rp_scene* s, rp_workspace* ws, const double* d_traces, int64_t ns, int form,
                    void* d_out, int64_t* counts, cudaStream_t st) {
    int f = form & 0xff;
    int out64 = (form & RP_OUT_COMPLEX128) ? 1 : 0;
    if (f == RP_FORM_PLAIN_F64) return rp_plain_run(s, ws, d_traces, ns, d_out, out64, counts, st);
    if (f == RP_FORM_FAST_F32) return rp_fast_run(s, ws, d_traces, ns, d_out, out64, counts, st);
    rp_set_error("unknown form %d", form);
    return RP_ERR_ARG;
}

extern "C" int rp_simulate_device(rp_scene* s, const double* d_traces, int64_t ns, int form,
                                  void* d_out, int64_t* counts, void* stream) {
    if (!s || ns < 0 || (ns > 0 && (!d_traces || !d_out))) {
        rp_set_error("rp_simulate_device: bad argument");
        return RP_ERR_ARG;
    }
    g_launches = 0;
    g_timer.reset();
    RP_CUDA(cudaSetDevice(s->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : s->own_stream;
    if (ns == 0) return RP_OK;
    return run_form(s, &s->ws, d_traces, ns, form, d_out, counts, st);
}

// ------------------------------------------------------------ graphs --
// A fast-form call (rp_graph_create) or batch (rp_graph_create_batch)
// recorded as a CUDA graph: planned from the host copy of its traces, its
// target windows sized by host bounds, run
// once eagerly (which reserves the buffers and tunes the pair kernel), then
// run again under stream capture into a graph that replays the whole call --
// setup, pair stage, compression, tails -- with one launch.  The graph owns
// its workspace (device buffers, auxiliary streams, the pinned staging of its
// job tables and of the flags and counts it reads back).
struct rp_graph {
    rp_workspace ws;
    cudaStream_t st = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t ns = 0;                                 // traces over all jobs
    std::vector<std::vector<double>> h_traces;      // per job: the host traces it was planned with
};

static void graph_release(rp_graph* g) {
    if (!g) return;
    cudaSetDevice(g->ws.device);
    cudaDeviceSynchronize();
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    g->ws.arena.release();
    g->ws.arena2.release();
    if (g->ws.aux_ready) {
        for (int k = 0; k < rp_workspace::kAux; ++k) {
            cudaStreamDestroy(g->ws.aux[k]);
            cudaEventDestroy(g->ws.ev_join[k]);
        }
        cudaEventDestroy(g->ws.ev_fork);
    }
    if (g->ws.pin) cudaFreeHost(g->ws.pin);
    if (g->st) cudaStreamDestroy(g->st);
    delete g;
}

// Records jobs (planned from g's host trace copies) on g's stream: the eager
// call first (buffers, tuning and every check of a plain call), then the same
// call under stream capture, instantiated.
static int graph_record(rp_graph* g, const std::vector<rp_job>& jobs, int64_t ns_total) {
    int rc = RP_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking);
    const size_t pin_bytes = ((size_t)4 << 20) + 16 * (size_t)ns_total + 4096 * jobs.size();
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&g->ws.pin, pin_bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) return rp_cuda_fail(e, "rp_graph_create");
    g->ws.pin_cap = pin_bytes;
    const int timing = g_timer.enabled;
    g->ws.graph_mode = 1;
    g_timer.enabled = 0;
    rc = rp_fast_batch(jobs.data(), (int)jobs.size(), &g->ws, g->st);
    if (!rc && (e = cudaStreamSynchronize(g->st)) != cudaSuccess) rc = rp_cuda_fail(e, "rp_graph_create");
    if (!rc) {
        g->ws.graph_mode = 2;
        g->ws.pin_off = 0;
        g->ws.graph_rb.clear();
        e = cudaStreamBeginCapture(g->st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            rc = rp_cuda_fail(e, "rp_graph_create: begin capture");
        } else {
            rc = rp_fast_batch(jobs.data(), (int)jobs.size(), &g->ws, g->st);
            e = cudaStreamEndCapture(g->st, &g->graph);
            if (!rc && e != cudaSuccess) rc = rp_cuda_fail(e, "rp_graph_create: end capture");
        }
        if (!rc && (e = cudaGraphInstantiate(&g->exec, g->graph, 0)) != cudaSuccess)
            rc = rp_cuda_fail(e, "rp_graph_create: instantiate");
    }
    g_timer.enabled = timing;
    return rc;
}

extern "C" int rp_graph_create(rp_scene* s, const double* h_traces, const double* d_traces, int64_t ns,
                               void* d_out, rp_graph** out) {
    if (!s || !h_traces || !d_traces || !d_out || !out || ns <= 0) {
        rp_set_error("rp_graph_create: bad argument");
        return RP_ERR_ARG;
    }
    *out = nullptr;
    RP_CUDA(cudaSetDevice(s->device));
    rp_graph* g = new rp_graph();
    g->ns = ns;
    g->ws.device = s->device;
    g->h_traces.assign(1, std::vector<double>(h_traces, h_traces + 9 * ns));
    g->ws.plan_traces = g->h_traces[0].data();
    const int rc = graph_record(g, std::vector<rp_job>{rp_job{s, d_traces, ns, d_out, nullptr}}, ns);
    if (rc) {
        cudaGetLastError();
        graph_release(g);
        return rc;
    }
    *out = g;
    return RP_OK;
}

extern "C" int rp_graph_create_batch(const rp_job* jobs, int njobs, const double* const* h_traces,
                                     rp_graph** out) {
    if (!jobs || njobs <= 0 || !h_traces || !out) {
        rp_set_error("rp_graph_create_batch: bad argument");
        return RP_ERR_ARG;
    }
    *out = nullptr;
    int64_t ns_total = 0;
    for (int j = 0; j < njobs; ++j) {
        const rp_job& b = jobs[j];
        if (!b.scene || b.ns <= 0 || !b.d_traces || !b.d_out || !h_traces[j] ||
            b.scene->device != jobs[0].scene->device) {
            rp_set_error("rp_graph_create_batch: job %d: bad scene, trace tables, output or device", j);
            return RP_ERR_ARG;
        }
        ns_total += b.ns;
    }
    RP_CUDA(cudaSetDevice(jobs[0].scene->device));
    rp_graph* g = new rp_graph();
    g->ns = ns_total;
    g->ws.device = jobs[0].scene->device;
    std::vector<rp_job> js(jobs, jobs + njobs);
    for (int j = 0; j < njobs; ++j) {
        js[j].counts = nullptr;         // rp_graph_check reports the counts
        g->h_traces.emplace_back(h_traces[j], h_traces[j] + 9 * jobs[j].ns);
    }
    for (const std::vector<double>& h : g->h_traces) g->ws.plan_jobs.push_back(h.data());
    const int rc = graph_record(g, js, ns_total);
    if (rc) {
        cudaGetLastError();
        graph_release(g);
        return rc;
    }
    *out = g;
    return RP_OK;
}

extern "C" int rp_graph_launch(rp_graph* g, void* stream) {
    if (!g || !g->exec) { rp_set_error("rp_graph_launch: null graph"); return RP_ERR_ARG; }
    RP_CUDA(cudaSetDevice(g->ws.device));
    RP_CUDA(cudaGraphLaunch(g->exec, stream ? (cudaStream_t)stream : g->st));
    return RP_OK;
}

extern "C" int rp_graph_check(const rp_graph* g, int64_t* counts) {
    if (!g) { rp_set_error("rp_graph_check: null graph"); return RP_ERR_ARG; }
    for (const rp_workspace::Readback& r : g->ws.graph_rb) {
        if (r.misc[6]) {
            rp_set_error("fast form: an illuminated-facet or target list exceeded its capacity (a replay's "
                         "traces outgrew the bounds the graph was planned with)");
            return RP_ERR_INTERNAL;
        }
        if (r.misc[3]) { rp_set_error("fast form: a shared-memory stage wait timed out"); return RP_ERR_TIMEOUT; }
        if (r.misc[2]) {
            rp_set_error("fast form: a pair fell outside its target's bin window (a replay's traces outgrew "
                         "the bounds the graph was planned with)");
            return RP_ERR_INTERNAL;
        }
        if (counts)
            for (int k = 0; k < r.nb; ++k) {
                counts[2 * (r.s0 + k)] = r.cnt[k];
                counts[2 * (r.s0 + k) + 1] = r.cnt[r.nb + k];
            }
    }
    return RP_OK;
}

extern "C" int rp_graph_destroy(rp_graph* g) {
    graph_release(g);
    return RP_OK;
}

int rp_workspace::ensure_aux() {
    if (aux_ready) return RP_OK;
    for (int k = 0; k < kAux; ++k) {
        RP_CUDA(cudaStreamCreateWithFlags(&aux[k], cudaStreamNonBlocking));
        RP_CUDA(cudaEventCreateWithFlags(&ev_join[k], cudaEventDisableTiming));
    }
    RP_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    aux_ready = true;
    return RP_OK;
}

void rp_workspace::fork(cudaStream_t st) {
    cudaEventRecord(ev_fork, st);
    for (int k = 0; k < kAux; ++k) cudaStreamWaitEvent(aux[k], ev_fork, 0);
}

void rp_workspace::join(cudaStream_t st) {
    for (int k = 0; k < kAux; ++k) {
        cudaEventRecord(ev_join[k], aux[k]);
        cudaStreamWaitEvent(st, ev_join[k], 0);
    }
}

extern "C" int rp_workspace_create(int device, rp_workspace** out) {
    if (!out) { rp_set_error("rp_workspace_create: null argument"); return RP_ERR_ARG; }
    *out = new rp_workspace();
    (*out)->device = device;
    return RP_OK;
}

extern "C" int rp_workspace_destroy(rp_workspace* ws) {
    if (!ws) return RP_OK;
    cudaSetDevice(ws->device);
    cudaDeviceSynchronize();
    ws->arena.release();
    ws->arena2.release();
    if (ws->aux_ready) {
        for (int k = 0; k < rp_workspace::kAux; ++k) {
            cudaStreamDestroy(ws->aux[k]);
            cudaEventDestroy(ws->ev_join[k]);
        }
        cudaEventDestroy(ws->ev_fork);
    }
    delete ws;
    return RP_OK;
}

extern "C" int rp_workspace_bytes(const rp_workspace* ws, int64_t* bytes) {
    if (!ws || !bytes) { rp_set_error("rp_workspace_bytes: null argument"); return RP_ERR_ARG; }
    *bytes = (int64_t)(ws->arena.cap + ws->arena2.cap);
    return RP_OK;
}

extern "C" int rp_simulate_ws(rp_scene* s, rp_workspace* ws, const double* d_traces, int64_t ns, int form,
                              void* d_out, int64_t* counts, void* stream) {
    if (!s || !ws || ns < 0 || (ns > 0 && (!d_traces || !d_out)) || ws->device != s->device) {
        rp_set_error("rp_simulate_ws: bad argument (scene and workspace must share a device)");
        return RP_ERR_ARG;
    }
    g_launches = 0;
    g_timer.reset();
    RP_CUDA(cudaSetDevice(s->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : s->own_stream;
    if (ns == 0) return RP_OK;
    return run_form(s, ws, d_traces, ns, form, d_out, counts, st);
}

extern "C" int rp_simulate_batch(const rp_job* jobs, int njobs, rp_workspace* ws, void* stream) {
    if (!ws || njobs < 0 || (njobs > 0 && !jobs)) {
        rp_set_error("rp_simulate_batch: bad argument");
        return RP_ERR_ARG;
    }
    g_launches = 0;
    g_timer.reset();
    std::vector<rp_job> live;
    for (int j = 0; j < njobs; ++j) {
        const rp_job& b = jobs[j];
        if (!b.scene || b.ns < 0 || (b.ns > 0 && (!b.d_traces || !b.d_out)) || b.scene->device != ws->device) {
            rp_set_error("rp_simulate_batch: job %d: bad scene, trace table, output or device", j);
            return RP_ERR_ARG;
        }
        if (b.ns > 0) live.push_back(b);
    }
    RP_CUDA(cudaSetDevice(ws->device));
    if (live.empty()) return RP_OK;
    cudaStream_t st = stream ? (cudaStream_t)stream : live[0].scene->own_stream;
    return rp_fast_batch(live.data(), (int)live.size(), ws, st);
}

extern "C" int rp_simulate(rp_scene* s, const double* traces, int64_t ns, int form, void* out,
                           int out_on_device, int64_t* counts, void* stream) {
    if (!s || ns < 0 || (ns > 0 && (!traces || !out))) {
        rp_set_error("rp_simulate: bad argument");
        return RP_ERR_ARG;
    }
    g_launches = 0;
    g_timer.reset();
    RP_CUDA(cudaSetDevice(s->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : s->own_stream;
    if (ns == 0) return RP_OK;
    const size_t esz = (form & RP_OUT_COMPLEX128) ? 16 : 8;
    const size_t out_bytes = esz * (size_t)s->nr * ns;
    double* d_tr = nullptr;
    void* d_out = out_on_device ? out : nullptr;
    RP_CUDA(cudaMallocAsync((void**)&d_tr, sizeof(double) * 9 * ns, st));
    if (!out_on_device) {
        cudaError_t e = cudaMallocAsync(&d_out, out_bytes, st);
        if (e != cudaSuccess) { cudaFreeAsync(d_tr, st); return rp_cuda_fail(e, "cudaMallocAsync(out)"); }
    }
    int rc = RP_OK;
    cudaError_t e = cudaMemcpyAsync(d_tr, traces, sizeof(double) * 9 * ns, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) rc = rp_cuda_fail(e, "cudaMemcpyAsync(traces)");
    if (rc == RP_OK) rc = run_form(s, &s->ws, d_tr, ns, form, d_out, counts, st);
    if (rc == RP_OK && !out_on_device) {
        e = cudaMemcpyAsync(out, d_out, out_bytes, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) rc = rp_cuda_fail(e, "cudaMemcpyAsync(out)");
    }
    cudaFreeAsync(d_tr, st);
    if (!out_on_device) cudaFreeAsync(d_out, st);
    e = cudaStreamSynchronize(st);
    if (rc == RP_OK && e != cudaSuccess) rc = rp_cuda_fail(e, "cudaStreamSynchronize");
    return rc;
}
