/*
 * oracle.cpp -- FP64 CPU restatement of the reference simulator's trace loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the correctness oracle and the timed CPU
 * baseline; the product library (libraypath.so) never links or calls it.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 *
 * It follows the reference (Nacnud04/EuropaRaypaths, src/CUDA/) line by line
 * for the default mode written by param_gen.gen_params (non-specular,
 * convolution, linear convolution), including attenuation prisms, lossless,
 * disable_surface and ttype 0 targets, and for the specular variants the
 * reference defines: specular with linear convolution (all target types),
 * specular without convolution and specular with circular convolution (ttype
 * 0 targets only: for other targets the reference uses buffers it never
 * allocates, sim.cu:411-445, 864-872).  Each function cites the reference
 * file:line it restates.  Deviations, all documented in the design notes:
 *   * the aperture test clamps the cosine to [-1, 1] before acos (the
 *     reference's unclamped acosf turns rounding above 1 into NaN and drops
 *     that facet, geometry_kernels.cu:95);
 *   * the second bin of the two-bin split is dropped when it equals nr (the
 *     reference writes one element past its buffer, radar_kernels.cu:757);
 *   * the accumulation order is the facet order (the reference uses float
 *     atomics, whose order is unspecified);
 *   * FFTs are this file's own FP64 radix-2 / Bluestein transforms with the
 *     cuFFT sign and scaling conventions (forward e^{-i}, inverse unscaled).
 *
 * Parallelism: OpenMP over targets (each target's two legs and convolutions
 * are independent); per-target results are summed in target order, so the
 * output does not depend on the thread count.
 */
#include "../include/raypath.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <mutex>
#include <map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using cd = std::complex<double>;

namespace {

const double PI_F = 3.14159265;   // geometry_kernels.cu:45, radar_kernels.cu:682
const double PI_FRIIS = 3.14159;  // geometry_kernels.cu:411, file_io.cu:196

// elementary_kernels.cu:50-53
inline double sinc(double x) {
    if (std::fabs(x) < 1e-6) return 1.0;
    return std::sin(M_PI * x) / (M_PI * x);
}

// radar_kernels.cu:658-677 (pi appears twice in the sinc argument)
inline double facet_G(double th, double ph, double lam, double fs) {
    double piLlam = (PI_F * fs) / lam;
    double s1 = sinc(piLlam * std::sin(th) * std::cos(ph));
    double s2 = sinc(piLlam * std::sin(th) * std::sin(ph));
    double D = (s1 * s2) * (s1 * s2);
    return D * (4 * PI_F * fs * fs) / (lam * lam);
}

// geometry_kernels.cu:410-412
inline double friis(double P, double Gt, double Gr, double lam, double d) {
    return (P * lam * lam * Gt * Gr) / ((4 * PI_FRIIS) * (4 * PI_FRIIS) * d * d);
}

// geometry_kernels.cu:384-393
inline double radar_eq(double P, double G, double fs, double lam, double d, double nf) {
    double num = P * G * G * fs * fs * fs * fs;
    double den = (4 * PI_FRIIS) * (4 * PI_FRIIS) * d * d * d * d;
    return nf * (num / den);
}

// radar_kernels.cu:681-686
// Incoherent mode's seeded surface phase in turns (the reference draws it
// from clock64(), radar_kernels.cu:689-711): the SplitMix64 mixing function
// over (seed, the source position's bits, the facet's input index), top 24
// bits.
inline uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
inline uint64_t dbits(double v) {
    uint64_t u;
    std::memcpy(&u, &v, sizeof(u));
    return u;
}
inline double inc_turns(uint64_t seed, double sx, double sy, double sz, int64_t i) {
    const uint64_t key = mix64(mix64(mix64(mix64(seed) ^ dbits(sx)) ^ dbits(sy)) ^ dbits(sz));
    return (double)(mix64(key ^ (uint64_t)i) >> 40) / 16777216.0;
}

inline cd phasor(double r, double lam) {
    double ph = -(2.0 * PI_F / lam) * r;
    return cd(std::cos(ph), std::sin(ph));
}

// radar_kernels.cu:167-189
inline double rerad(int f, double th1) {
    switch (f) {
        case 0: return 1.0;
        case 1: return th1 * (180 / PI_F) < 1 ? 1.0 : 0.0;
        case 2: return th1 * (180 / PI_F) < 0.5 ? 1.0 : 0.0;
        case 3: return th1 * (PI_F / 180) < 3 ? 1.0 : 0.0;
        case 4: { double s = PI_F / 180; return std::exp(-0.5 * th1 * th1 / (s * s)); }
        default: return 1.0;
    }
}

inline double clamp1(double x) { return std::max(-1.0, std::min(1.0, x)); }

// facetReradiation, geometry_kernels.cu:353-381 (sinc arguments without pi)
inline double facet_rerad(double th, double ph, double lam, double fs) {
    double s1 = sinc((fs / lam) * std::sin(th) * std::cos(ph));
    double s2 = sinc((fs / lam) * std::sin(th) * std::sin(ph));
    double v = (fs * fs / lam) * s1 * s2;
    return v * v;
}

// snellsLaw, geometry_kernels.cu:490-501 (1e4 flags total internal reflection)
inline double snells(double th, double e1, double e2) {
    double sR = std::sqrt(e1 / e2) * std::sin(th);
    return sR > 1.0 ? 1e4 : std::asin(sR);
}

// Two-bin linear split of surfacePT / accumulateTarget / radiateTarget,
// radar_kernels.cu:736-760: bin = (short)x (truncation), w = x - bin.
inline void split_add(cd* tr, int nr, double x, cd v) {
    if (!(x > -1.0) || x >= (double)nr) return;   // trunc(x) outside [0, nr)
    long b = (long)x;                               // truncation toward zero
    double w = x - (double)b;
    tr[b] += v * (1.0 - w);
    if (b + 1 < nr) tr[b + 1] += v * w;
}

// prismIntersectionDistance, geometry_kernels.cu:207-269
double prism_dist(const double o[3], const double d[3], const double box[6], double t) {
    const double INF = 1e30;
    double lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        double mn = box[a], mx = box[a + 3];
        if (std::fabs(d[a]) < 1e-12) {
            if (o[a] < mn || o[a] > mx) return 0.0;
            lo[a] = -INF; hi[a] = INF;
        } else {
            double t1 = (mn - o[a]) / d[a], t2 = (mx - o[a]) / d[a];
            if (t1 > t2) std::swap(t1, t2);
            lo[a] = t1; hi[a] = t2;
        }
    }
    double te = std::max(std::max(lo[0], lo[1]), lo[2]);
    double tx = std::min(std::min(hi[0], hi[1]), hi[2]);
    if (te < 0.0) te = 0.0;
    if (tx > t) tx = t;
    if (te >= tx) return 0.0;
    return tx - te;
}

// ---------------------------------------------------------------- FFT ----
// In-place iterative radix-2 FFT; sign = -1 forward (e^{-i}), +1 inverse
// (unscaled), the cuFFT conventions used by the reference.
void fft_pow2(cd* a, int n, int sign) {
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(a[i], a[j]);
    }
    for (int len = 2; len <= n; len <<= 1) {
        double ang = sign * 2.0 * M_PI / len;
        int half = len >> 1;
        for (int k = 0; k < half; ++k) {
            cd w(std::cos(ang * k), std::sin(ang * k));
            for (int i = 0; i < n; i += len) {
                cd u = a[i + k], v = a[i + k + half] * w;
                a[i + k] = u + v;
                a[i + k + half] = u - v;
            }
        }
    }
}

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// Bluestein plan for an arbitrary length n (chirp-z with a power-of-two m).
struct Blue {
    int n = 0, m = 0;
    std::vector<cd> w;      // w_k = exp(-i pi k^2 / n)
    std::vector<cd> Wf;     // FFT_m of conj chirp b_k = conj(w_k) (k and m-k)
};

std::mutex g_blue_mu;
std::map<int, Blue*> g_blue;

const Blue* blue_plan(int n) {
    std::lock_guard<std::mutex> lk(g_blue_mu);
    auto it = g_blue.find(n);
    if (it != g_blue.end()) return it->second;
    Blue* b = new Blue;
    b->n = n;
    int m = 1;
    while (m < 2 * n - 1) m <<= 1;
    b->m = m;
    b->w.resize(n);
    for (int k = 0; k < n; ++k) {
        long long kk = ((long long)k * k) % (2LL * n);   // exact angle reduction
        double ang = -M_PI * (double)kk / n;
        b->w[k] = cd(std::cos(ang), std::sin(ang));
    }
    b->Wf.assign(m, cd(0, 0));
    for (int k = 0; k < n; ++k) {
        b->Wf[k] = std::conj(b->w[k]);
        if (k) b->Wf[m - k] = std::conj(b->w[k]);
    }
    fft_pow2(b->Wf.data(), m, -1);
    g_blue[n] = b;
    return b;
}

// DFT of any length with the cuFFT conventions; work must hold m entries.
void dft(cd* a, int n, int sign, std::vector<cd>& work) {
    if (is_pow2(n)) { fft_pow2(a, n, sign); return; }
    const Blue* b = blue_plan(n);
    int m = b->m;
    work.assign(m, cd(0, 0));
    // forward uses w; inverse uses conj(w): e^{+i 2pi jk/n} chirp
    for (int k = 0; k < n; ++k) {
        cd wk = sign < 0 ? b->w[k] : std::conj(b->w[k]);
        work[k] = a[k] * wk;
    }
    fft_pow2(work.data(), m, -1);
    if (sign < 0) {
        for (int k = 0; k < m; ++k) work[k] *= b->Wf[k];
    } else {
        // chirp conj(conj(w)) = w: FFT of w sequence = conj-symmetric of Wf
        // FFT_m(w)[k] = conj(FFT_m(conj w)[(m-k) % m])
        for (int k = 0; k < m; ++k) work[k] *= std::conj(b->Wf[(m - k) % m]);
    }
    fft_pow2(work.data(), m, +1);
    double inv = 1.0 / m;
    for (int k = 0; k < n; ++k) {
        cd wk = sign < 0 ? b->w[k] : std::conj(b->w[k]);
        a[k] = work[k] * inv * wk;
    }
}

// genCenteredChirpPadded, radar_kernels.cu:489-503 (length 2 nr), already
// transformed: returns FFT_2nr of the real chirp.
std::vector<cd> chirp_spectrum(int nr, double dr, double res) {
    std::vector<cd> c(2 * nr), work;
    for (int i = 0; i < 2 * nr; ++i) c[i] = cd(sinc((double)(i - nr / 2) * dr / res), 0.0);
    dft(c.data(), 2 * nr, -1, work);
    return c;
}

// genChirp, radar_kernels.cu:454-466: the sinc at the window start plus its
// wrap at rst + nr dr, i.e. sinc(i dr / res) + sinc((i - nr) dr / res),
// already transformed: returns DFT_nr of the real chirp.
std::vector<cd> chirp_wrapped_spectrum(int nr, double dr, double res) {
    std::vector<cd> c(nr), work;
    for (int i = 0; i < nr; ++i)
        c[i] = cd(sinc((double)i * dr / res) + sinc((double)(i - nr) * dr / res), 0.0);
    dft(c.data(), nr, -1, work);
    return c;
}

// convolvePhasorChirp, radar_kernels.cu:516-552: circular convolution of
// length nr, scaled 1/nr.
void conv_circular(const cd* tr, const std::vector<cd>& C, int nr, cd* out, std::vector<cd>& buf,
                   std::vector<cd>& work) {
    buf.assign(tr, tr + nr);
    dft(buf.data(), nr, -1, work);
    for (int i = 0; i < nr; ++i) buf[i] *= C[i];
    dft(buf.data(), nr, +1, work);
    for (int i = 0; i < nr; ++i) out[i] = buf[i] / (double)nr;
}

// convolvePhasorChirpLinear, radar_kernels.cu:554-649:
// pad to 2nr, multiply spectra, inverse, scale 1/(2nr), window at nr/2.
void conv_linear(const cd* tr, const std::vector<cd>& C, int nr, cd* out, std::vector<cd>& buf,
                 std::vector<cd>& work) {
    int n2 = 2 * nr;
    buf.assign(n2, cd(0, 0));
    for (int i = 0; i < nr; ++i) buf[i] = tr[i];
    dft(buf.data(), n2, -1, work);
    for (int i = 0; i < n2; ++i) buf[i] *= C[i];
    dft(buf.data(), n2, +1, work);
    double sc = 1.0 / n2;
    for (int i = 0; i < nr; ++i) out[i] = buf[nr / 2 + i] * sc;
}

// convolveComplex + cropSpectrum + takeEveryOtherComplex,
// elementary_kernels.cu:258-353 and :187-194, at N = 2 nr - 1.
void conv_complex(const cd* sig, const cd* ker, int nr, double smpl, double B,
                  cd* out, std::vector<cd>& a, std::vector<cd>& b, std::vector<cd>& work) {
    int N = 2 * nr - 1;
    a.assign(N, cd(0, 0));
    b.assign(N, cd(0, 0));
    for (int i = 0; i < nr; ++i) { a[i] = sig[i]; b[i] = ker[i]; }
    dft(a.data(), N, -1, work);
    dft(b.data(), N, -1, work);
    for (int k = 0; k < N; ++k) {
        double f = (k <= N / 2) ? (double)k * smpl / N : (double)(k - N) * smpl / N;
        if (std::fabs(f) > B) b[k] = 0.0;
        a[k] *= b[k];
    }
    dft(a.data(), N, +1, work);
    double sc = 1.0 / N;
    for (int k = 0; k < nr; ++k) out[k] = a[2 * k] * sc;
}

}  // namespace

extern "C" {

/* Restatement of parseSimulationParameters' derivations, file_io.cu:167-213,
 * in FP64; nr follows the float expression of file_io.cu:212 exactly. */
int oracle_params_derive(rp_params* p) {
    double c = 299792458.0;
    p->c = c;
    p->rng_res = c / p->bandwidth;
    p->lam = c / p->frequency;
    p->k = 2 * PI_F / p->lam;
    p->grefr_lin = std::pow(10.0, p->subsurface_gain / 10.0);
    p->grefl_lin = std::pow(10.0, p->surface_gain / 10.0);
    p->ks = p->k * p->rms_height;
    p->c_1 = c / std::sqrt(p->eps_1);
    p->c_2 = c / std::sqrt(p->eps_2);
    p->nu_1 = 376.7 / std::sqrt(p->eps_1);
    p->nu_2 = 376.7 / std::sqrt(p->eps_2);
    auto alpha = [&](double sig, double eps) {
        double epp = sig / (2 * PI_FRIIS * p->frequency * 8.85e-12);
        double a = std::sqrt(1 + (epp / eps) * (epp / eps)) - 1;
        a = std::sqrt(0.5 * eps * a);
        return (a * 2 * PI_FRIIS) / p->lam;
    };
    p->alpha1 = alpha(p->sig_1, p->eps_1);
    p->alpha2 = alpha(p->sig_2, p->eps_2);
    float nrf = ((float)p->rx_window_m / 299792480.0f) * (float)p->rx_sample_rate;
    p->nr = (int32_t)nrf;
    if (p->nr <= 0) return RP_ERR_ARG;
    p->dr = p->rx_window_m / (double)p->nr;
    return RP_OK;
}

/*
 * Run the trace loop of src/CUDA/sim.cu:615-1008 in FP64.
 *   facets [12][nf], targets [7][nt], prisms [7][np] (alpha already), traces
 *   [ns][9]; out double[ns][nr][2]; counts int64[ns][2] (may be NULL).
 *   max_targets: if > 0, only the first max_targets in-aperture targets of
 *   each trace are processed (bounded CPU-baseline samples).
 */
int oracle_simulate(const rp_params* P, const double* facets, int64_t nf,
                    const double* targets, int64_t nt, const double* prisms, int64_t np,
                    const double* traces, int64_t ns, double* out, int64_t* counts,
                    int nthreads, int64_t max_targets) {
    const rp_params& p = *P;
    const int nr = p.nr;
    const double dr = p.dr, lam = p.lam, fs = p.fs;
    const double ap = p.aperture * (M_PI / 180.0);
    const double nidx = std::sqrt(p.eps_2);
    if (nr <= 0 || nf < 0 || nt < 0 || ns < 0) return RP_ERR_ARG;
    // mode (sim.cu:733-986): conv mode 0 linear, 1 circular, 2 none
    const bool spec = p.specular != 0;
    const int cmode = !p.convolution ? 2 : (p.convolution_linear ? 0 : 1);
    if (!spec && cmode != 0) return RP_ERR_UNSUPPORTED;   // chirp written past its buffer (sim.cu:431-438, 851-856)
    if (spec && cmode != 0)
        for (int64_t t = 0; t < nt; ++t)
            if (targets[6 * nt + t] != 0.0) return RP_ERR_UNSUPPORTED;   // unallocated chirp / temp buffer
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    const double* FX = facets;
    auto F = [&](int c, int64_t i) { return FX[(int64_t)c * nf + i]; };
    auto TG = [&](int c, int64_t i) { return targets[(int64_t)c * nt + i]; };
    auto PR = [&](int c, int64_t i) { return prisms[(int64_t)c * np + i]; };

    std::vector<cd> C1 = chirp_spectrum(nr, dr, p.rng_res);
    std::vector<cd> C2 = chirp_spectrum(nr, dr, 2 * p.rng_res);
    // specular mode never regenerates the chirp: targets use C1 (sim.cu:851-856)
    const std::vector<cd>& CT = spec ? C1 : C2;
    std::vector<cd> CR;
    if (cmode == 1) CR = chirp_wrapped_spectrum(nr, dr, p.rng_res);
    std::memset(out, 0, sizeof(double) * 2 * nr * ns);

    std::vector<int64_t> ill;
    std::vector<double> Itd, Ith, Iph, Rth, fRe, fRfrC, Gi, fx, fy, fz;
    for (int64_t s = 0; s < ns; ++s) {
        const double* tr = traces + 9 * s;
        const double sx = tr[0], sy = tr[1], sz = tr[2];
        const double snx = tr[3], sny = tr[4], snz = tr[5];
        const double rst = tr[6], grefl = tr[7], grefr = tr[8];
        // compSourceInclination + cropByAperture, geometry_kernels.cu:75-204
        ill.clear();
        for (int64_t i = 0; i < nf; ++i) {
            double dx = F(0, i) - sx, dy = F(1, i) - sy, dz = F(2, i) - sz;
            double d = std::sqrt(dx * dx + dy * dy + dz * dz);
            double cs = clamp1((-dx / d) * snx + (-dy / d) * sny + (-dz / d) * snz);
            if (std::acos(cs) < ap) ill.push_back(i);
        }
        const int64_t nv = (int64_t)ill.size();
        if (counts) { counts[2 * s] = nv; counts[2 * s + 1] = 0; }
        if (nv == 0) continue;   // sim.cu:693-697
        Itd.resize(nv); Ith.resize(nv); Iph.resize(nv); Rth.resize(nv);
        fRe.resize(nv); fRfrC.resize(nv); Gi.resize(nv);
        fx.resize(nv); fy.resize(nv); fz.resize(nv);
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < nv; ++j) {
            int64_t i = ill[j];
            // compIncidentRays, geometry_kernels.cu:103-140
            double dx = F(0, i) - sx, dy = F(1, i) - sy, dz = F(2, i) - sz;
            double d = std::sqrt(dx * dx + dy * dy + dz * dz);
            double Ix = dx / d, Iy = dy / d, Iz = dz / d;
            double th = std::acos(clamp1(-Ix * F(3, i) - Iy * F(4, i) - Iz * F(5, i)));
            double ph = std::atan2(Ix * F(6, i) + Iy * F(7, i) + Iz * F(8, i),
                                   Ix * F(9, i) + Iy * F(10, i) + Iz * F(11, i));
            // snellsLaw, geometry_kernels.cu:490-501
            double sR = std::sqrt(p.eps_1 / p.eps_2) * std::sin(th);
            double rth = sR > 1.0 ? 1e4 : std::asin(sR);
            // compReflectedEnergy (non-specular, H pol), geometry_kernels.cu:426-487
            double cI = std::cos(th), cR = std::cos(rth);
            double rho = (p.nu_2 * cI - p.nu_1 * cR) / (p.nu_2 * cI + p.nu_1 * cR);
            double frc = 1.0 - rho * rho;
            // specular: facetReradiation at twice the inclination times the
            // radar equation (geometry_kernels.cu:434-446); else 1
            double fre = spec ? facet_rerad(2 * th, -ph, lam, fs) * radar_eq(p.power, grefl, fs, lam, d, (double)nv)
                              : 1.0;
            fre *= rho * rho;
            if (rth > 1e3) frc = 0.0;
            double atm = std::exp(-4.0 * p.alpha1 * d);
            fre *= atm; frc *= atm;
            fre *= std::exp(-4 * ((p.ks * cI) * (p.ks * cI)));
            Itd[j] = d; Ith[j] = th; Iph[j] = ph; Rth[j] = rth; fRe[j] = fre; fRfrC[j] = frc;
            Gi[j] = facet_G(th, ph, lam, fs);
            fx[j] = F(0, i); fy[j] = F(1, i); fz[j] = F(2, i);
        }
        std::vector<cd> refl(nr, cd(0, 0)), buf, wk;
        if (!spec) {
            // surfacePT, radar_kernels.cu:714-764 (facet order)
            std::vector<cd> psurf(nr, cd(0, 0));
            for (int64_t j = 0; j < nv; ++j) {
                double Pf = friis(p.power, grefr, Gi[j], lam, Itd[j]);
                double Ps = friis(Pf, Gi[j], grefr, lam, Itd[j]);
                if (!p.lossless) Ps *= fRe[j];
                // incoherent mode: randomPhasor (radar_kernels.cu:741-742), seeded
                const cd ph = p.incoherent ? std::polar(1.0, 2.0 * M_PI * inc_turns((uint64_t)p.incoherent_seed,
                                                                                    sx, sy, sz, ill[j]))
                                           : phasor(2 * Itd[j], lam);
                split_add(psurf.data(), nr, (Itd[j] - rst) / dr, ph * std::sqrt(Ps));
            }
            if (p.disable_surface) std::fill(psurf.begin(), psurf.end(), cd(0, 0));
            conv_linear(psurf.data(), C1, nr, refl.data(), buf, wk);
        } else if (cmode == 0) {
            // genReflPhasor + genPhasorTrace (radar_kernels.cu:314-346, 407-451):
            // one truncated bin per facet, summed in facet order
            std::vector<cd> ptr(nr, cd(0, 0));
            for (int64_t j = 0; j < nv; ++j) {
                double x = (Itd[j] - rst) / dr;
                if (!(x > -1.0) || x >= (double)nr) continue;
                double ph4 = (4.0 * PI_F / lam) * Itd[j];
                ptr[(long)x] += cd(std::cos(ph4), std::sin(ph4)) * fRe[j];
            }
            conv_linear(ptr.data(), C1, nr, refl.data(), buf, wk);                     // sim.cu:770
        } else if (cmode == 2) {
            // reflRadarSignal, radar_kernels.cu:58-160 (facet order per bin)
            for (int ir = 0; ir < nr; ++ir) {
                cd acc(0, 0);
                for (int64_t j = 0; j < nv; ++j) {
                    double ph4 = (4.0 * PI_F / lam) * Itd[j];
                    acc += cd(std::cos(ph4), std::sin(ph4)) * (sinc((rst + ir * dr - Itd[j]) / p.rng_res) * fRe[j]);
                }
                refl[ir] = acc;
            }
        }   // circular: the reference's surface convolution is commented out (sim.cu:765-767)

        // target loop, sim.cu:801-986: aperture test on the host (:808-826)
        std::vector<int64_t> tl;
        for (int64_t t = 0; t < nt; ++t) {
            double vx = TG(0, t) - sx, vy = TG(1, t) - sy, vz = TG(2, t) - sz;
            double m = std::sqrt(vx * vx + vy * vy + vz * vz);
            double th = std::acos(clamp1(-snx * vx / m - sny * vy / m - snz * vz / m));
            if (th > ap) continue;
            tl.push_back(t);
            if (max_targets > 0 && (int64_t)tl.size() >= max_targets) break;
        }
        if (counts) counts[2 * s + 1] = (int64_t)tl.size();
        const int64_t ntl = (int64_t)tl.size();
        std::vector<cd> refr_all((size_t)ntl * nr);
#pragma omp parallel
        {
            std::vector<cd> pt(nr), ps(nr), ptarg(nr), b1, a2, b2, work;
            std::vector<double> drr, drg;     // direct-sum phasors (no convolution)
#pragma omp for schedule(dynamic, 1)
            for (int64_t q = 0; q < ntl; ++q) {
                int64_t t = tl[q];
                double tx = TG(0, t), ty = TG(1, t), tz = TG(2, t);
                double tnx = TG(3, t), tny = TG(4, t), tnz = TG(5, t);
                int ttype = (int)TG(6, t);
                std::fill(pt.begin(), pt.end(), cd(0, 0));
                std::fill(ps.begin(), ps.end(), cd(0, 0));
                drr.clear();
                drg.clear();
                for (int64_t j = 0; j < nv; ++j) {
                    int64_t i = ill[j];
                    // compTargetRays, geometry_kernels.cu:272-350
                    double dx = tx - fx[j], dy = ty - fy[j], dz = tz - fz[j];
                    double Ttd = std::sqrt(dx * dx + dy * dy + dz * dz);
                    double Jx = dx / Ttd, Jy = dy / Ttd, Jz = dz / Ttd;
                    double Tth = std::acos(clamp1(-Jx * F(3, i) - Jy * F(4, i) - Jz * F(5, i)));
                    double TarTh = std::acos(clamp1(-Jx * tnx - Jy * tny - Jz * tnz));
                    double Tph = std::atan2(Jx * F(6, i) + Jy * F(7, i) + Jz * F(8, i),
                                            Jx * F(9, i) + Jy * F(10, i) + Jz * F(11, i));
                    double expo = 0.0, tot = 0.0;
                    if (np > 0) {
                        double o[3] = {fx[j], fy[j], fz[j]}, dd[3] = {Jx, Jy, Jz};
                        for (int64_t k = 0; k < np; ++k) {
                            double box[6] = {PR(1, k), PR(2, k), PR(3, k), PR(4, k), PR(5, k), PR(6, k)};
                            double ad = prism_dist(o, dd, box, Ttd);
                            tot += ad;
                            expo += PR(0, k) * ad;
                        }
                    }
                    expo += p.alpha2 * (Ttd - tot);
                    double att = std::exp(-4 * expo);
                    // compRefrEnergyIn / compRefrEnergyOut, geometry_kernels.cu:520-584
                    double cT = std::cos(Tth);
                    double rough = std::exp(-4 * ((p.ks * cT) * (p.ks * cT)));
                    double fEI = att, fEO = att;
                    if (spec) {
                        fEI *= facet_rerad(Rth[j] - Tth, Iph[j] - Tph, lam, fs);          // :528-537
                        double RrTh = snells(PI_F - Tth, p.eps_2, p.eps_1);                // :565-570
                        fEO *= facet_rerad(RrTh, Tph - Iph[j], lam, fs);
                    }
                    fEI = fEI * fRfrC[j] * rough;
                    fEO = fEO * fRfrC[j] * rough;
                    double fSR = Itd[j] + Ttd;
                    if (ttype != 0) {
                        // accumulateTarget, radar_kernels.cu:767-830
                        double Gd = facet_G(TarTh, Tph, lam, fs);
                        double Gt = facet_G(Tth, Tph, lam, fs);
                        double Pin = friis(friis(p.power, grefr, Gi[j], lam, Itd[j]), Gt, Gd, lam, Ttd);
                        if (!p.lossless) Pin *= fEI;
                        double rngt = Itd[j] + Ttd * nidx;
                        double x = (rngt - rst) / dr;
                        split_add(pt.data(), nr, x, phasor(rngt, lam) * std::sqrt(Pin * nidx));
                        // radiateTarget, radar_kernels.cu:834-892
                        double Pout = friis(friis(1.0, grefr, Gi[j], lam, Itd[j]), Gt, Gd, lam, Ttd);
                        if (!p.lossless) Pout *= fEO;
                        split_add(ps.data(), nr, x, phasor(rngt - lam / 2.0, lam) * std::sqrt(Pout * nidx));
                    } else if (cmode == 2) {
                        // refrRadarSignal, radar_kernels.cu:201-300: rerad of the
                        // facet-frame angle Tth and c / c2 (the reference's arguments)
                        double rr = rerad(p.rerad_funct, Tth) * fEI * fEO;
                        rr *= radar_eq(p.power, grefr, fs, lam, fSR, (double)nv);
                        drr.push_back(rr);
                        drg.push_back((fSR - Ttd) + Ttd * (p.c / p.c_2));
                    } else {
                        // genRefrPhasor, radar_kernels.cu:351-398 (binned into ps)
                        double rr = rerad(p.rerad_funct, TarTh) * fEI * fEO;
                        rr *= radar_eq(p.power, grefr, fs, lam, fSR, (double)nv);
                        double rngt = (fSR - Ttd) + Ttd * (p.c_1 / p.c_2);
                        double ph4 = (4.0 * PI_F / lam) * rngt;
                        double x = (rngt - rst) / dr;
                        if (x > -1.0 && x < (double)nr) {
                            long b = (long)x;
                            ps[b] += cd(std::cos(ph4), std::sin(ph4)) * rr;
                        }
                    }
                }
                cd* dst = refr_all.data() + (size_t)q * nr;
                if (ttype != 0) {
                    conv_linear(pt.data(), CT, nr, ptarg.data(), b1, work);                 // sim.cu:872
                    conv_complex(ps.data(), ptarg.data(), nr, p.rx_sample_rate, p.bandwidth,
                                 dst, a2, b2, work);                                    // sim.cu:912
                } else if (cmode == 0) {
                    conv_linear(ps.data(), CT, nr, dst, b1, work);                          // sim.cu:963
                } else if (cmode == 1) {
                    conv_circular(ps.data(), CR, nr, dst, b1, work);                        // sim.cu:959
                } else {
                    for (int ir = 0; ir < nr; ++ir) {                                    // sim.cu:928-936
                        cd acc(0, 0);
                        for (size_t k = 0; k < drr.size(); ++k) {
                            double ph4 = (4.0 * PI_F / lam) * drg[k];
                            acc += cd(std::cos(ph4), std::sin(ph4)) *
                                   (sinc((rst + ir * dr - drg[k]) / p.rng_res) * drr[k]);
                        }
                        dst[ir] = acc;
                    }
                }
            }
        }
        double* o = out + (size_t)2 * nr * s;
        for (int i = 0; i < nr; ++i) {
            cd acc(0, 0);
            for (int64_t q = 0; q < ntl; ++q) acc += refr_all[(size_t)q * nr + i];  // sim.cu:980
            cd v = refl[i] + acc;                                                   // sim.cu:989
            o[2 * i] = v.real();
            o[2 * i + 1] = v.imag();
        }
    }
    return RP_OK;
}

}  // extern "C"
