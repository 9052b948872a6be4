// rp_plain.cu -- the plain FP64 form: a double-precision GPU restatement of
// the reference trace loop (src/CUDA/sim.cu:615-1008).  Both target legs
// (accumulateTarget, radiateTarget) are evaluated separately as the reference
// does; accumulation is deterministic (single-owner targets, fixed-point
// surface bins, fixed-order sums).  It is the comparison point of the fast
// form and the oracle for sizes the CPU cannot reach.
#include <algorithm>
#include <cmath>
#include <vector>

#include "rp_common.cuh"
#include "rp_conv.cuh"

namespace {

using C64 = Cx<double>;

// compIncidentRays + snellsLaw + compReflectedEnergy + the surface leg, per
// (trace, illuminated facet).  geometry_kernels.cu:103-140, 426-517.  The
// surface leg: surfacePT's two-bin phasor (non-specular, radar_kernels.cu:
// 714-764), genReflPhasor's one-bin phasor (specular with linear convolution,
// :314-346); the other specular modes keep (Itd, fRe) for reflRadarSignal.
__global__ void k_incident64(const double* __restrict__ F, int64_t nf, const int* __restrict__ idx,
                             const int* __restrict__ nill, const double* __restrict__ traces,
                             DevParams dp, double* __restrict__ Itd_o, double* __restrict__ Gi_o,
                             double* __restrict__ frc_o, double* __restrict__ sx_o,
                             C64* __restrict__ sv_o, unsigned long long* __restrict__ vmax,
                             double* __restrict__ Rth_o, double* __restrict__ Iph_o,
                             double* __restrict__ fre_o) {
    const int s = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nill[s]) return;
    const TraceRow t = load_trace(traces, s);
    const size_t o = (size_t)s * nf + j;
    const int64_t i = idx[o];
    double dx = F[i] - t.sx, dy = F[nf + i] - t.sy, dz = F[2 * nf + i] - t.sz;
    double d = sqrt(dx * dx + dy * dy + dz * dz);
    double Ix = dx / d, Iy = dy / d, Iz = dz / d;
    double th = acos(clamp1(-Ix * F[3 * nf + i] - Iy * F[4 * nf + i] - Iz * F[5 * nf + i]));
    double ph = atan2(Ix * F[6 * nf + i] + Iy * F[7 * nf + i] + Iz * F[8 * nf + i],
                      Ix * F[9 * nf + i] + Iy * F[10 * nf + i] + Iz * F[11 * nf + i]);
    double sR = sqrt(dp.eps1 / dp.eps2) * sin(th);
    double rth = sR > 1.0 ? 1e4 : asin(sR);
    double cI = cos(th), cR = cos(rth);
    double rho = (dp.nu2 * cI - dp.nu1 * cR) / (dp.nu2 * cI + dp.nu1 * cR);
    double frc = 1.0 - rho * rho;
    // specular: facetReradiation at twice the inclination times the radar
    // equation (geometry_kernels.cu:434-446); non-specular: 1
    double fre = dp.specular ? d_facet_rerad(2 * th, -ph, dp.lam, dp.fs) *
                                   d_radar_eq(dp.P, t.grefl, dp.fs, dp.lam, d, (double)nill[s])
                             : 1.0;
    fre *= rho * rho;
    if (rth > 1e3) frc = 0.0;
    double atm = exp(-4.0 * dp.alpha1 * d);
    fre *= atm;
    frc *= atm;
    fre *= exp(-4 * ((dp.ks * cI) * (dp.ks * cI)));
    double G = d_facet_G(th, ph, dp.lam, dp.fs);
    Itd_o[o] = d;
    Gi_o[o] = G;
    frc_o[o] = frc;
    Rth_o[o] = rth;
    Iph_o[o] = ph;
    fre_o[o] = fre;
    if (dp.specular) {
        if (dp.cmode == 0) {
            // genReflPhasor: fRe e^{+j 4 pi_F Itd / lam} at bin (short)((Itd - rst)/dr)
            double sn, cs;
            sincos((4.0 * RP_PI_F / dp.lam) * d, &sn, &cs);
            sx_o[o] = (d - t.rst) / dp.dr;
            sv_o[o] = C64{fre * cs, fre * sn};
            atomic_max_pos(vmax + s, fabs(fre));
        } else {
            sx_o[o] = -2.0;          // no binned surface trace in these modes
            sv_o[o] = C64{0.0, 0.0};
        }
        return;
    }
    // surfacePT: two Friis hops with the subsurface gain (radar_kernels.cu:722-733)
    double Pf = d_friis(dp.P, t.grefr, G, dp.lam, d);
    double Ps = d_friis(Pf, G, t.grefr, dp.lam, d);
    if (!dp.lossless) Ps *= fre;
    double amp = sqrt(Ps);
    double sn, cs;
    if (dp.incoherent) {        // randomPhasor (radar_kernels.cu:741-742), seeded
        sincospi(2.0 * rp_incoherent_turns(dp.inc_seed, t.sx, t.sy, t.sz, i), &sn, &cs);
    } else {
        double phs = -(2.0 * RP_PI_F / dp.lam) * (2 * d);
        sincos(phs, &sn, &cs);
    }
    sx_o[o] = (d - t.rst) / dp.dr;
    sv_o[o] = C64{amp * cs, amp * sn};
    atomic_max_pos(vmax + s, amp);
}

// Fixed-point accumulation of the surface leg into acc[s][nr][2].
// single: one truncated bin per facet (genPhasorTrace) instead of the split.
__global__ void k_surf_fix64(int64_t nf, const int* __restrict__ nill, const double* __restrict__ sx,
                             const C64* __restrict__ sv, const unsigned long long* __restrict__ vmax,
                             int nr, long long* __restrict__ acc, int single) {
    const int s = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = nill[s];
    if (j >= n) return;
    double vm = __longlong_as_double((long long)vmax[s]);
    if (!(vm > 0)) return;
    const double scale = ldexp(1.0, RP_FIX_BITS) / (2.0 * (double)n * vm);
    const size_t o = (size_t)s * nf + j;
    double x = sx[o];
    if (!(x > -1.0) || x >= (double)nr) return;
    long b = (long)x;
    double w = x - (double)b;
    C64 v = sv[o];
    long long* a = acc + (size_t)s * nr * 2;
    if (single) {
        fix_add(a + 2 * b, v.x, scale);
        fix_add(a + 2 * b + 1, v.y, scale);
        return;
    }
    fix_add(a + 2 * b, v.x * (1.0 - w), scale);
    fix_add(a + 2 * b + 1, v.y * (1.0 - w), scale);
    if (b + 1 < nr) {
        fix_add(a + 2 * (b + 1), v.x * w, scale);
        fix_add(a + 2 * (b + 1) + 1, v.y * w, scale);
    }
}

// Both target legs for one (trace, in-aperture target) per thread.
// compTargetRays, compRefrEnergyIn/Out (geometry_kernels.cu:272-350,
// 520-584), accumulateTarget / radiateTarget (radar_kernels.cu:767-892) and,
// for ttype 0 targets, genRefrPhasor (radar_kernels.cu:351-398).
__global__ void k_pairs64(const double* __restrict__ F, int64_t nf, const int* __restrict__ idx,
                          const int* __restrict__ nill, const double* __restrict__ TG, int64_t nt,
                          const int* __restrict__ tlist, const int* __restrict__ ntl,
                          int64_t tstride, const double* __restrict__ PR, int64_t np,
                          const double* __restrict__ traces, DevParams dp,
                          const double* __restrict__ Itd, const double* __restrict__ Gi,
                          const double* __restrict__ frc, C64* __restrict__ PT,
                          C64* __restrict__ PS, const double* __restrict__ Rth,
                          const double* __restrict__ Iph, double2* __restrict__ PD) {
    const int s = blockIdx.y;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ntl[s]) return;
    const TraceRow t = load_trace(traces, s);
    const int nr = dp.nr;
    const int64_t ti = tlist[(size_t)s * tstride + q];
    const double tx = TG[ti], ty = TG[nt + ti], tz = TG[2 * nt + ti];
    const double tnx = TG[3 * nt + ti], tny = TG[4 * nt + ti], tnz = TG[5 * nt + ti];
    const int ttype = (int)TG[6 * nt + ti];
    C64* pt = PT + ((size_t)s * tstride + q) * nr;
    C64* ps = PS + ((size_t)s * tstride + q) * nr;
    const int nv = nill[s];
    const double rst = t.rst, grefr = t.grefr, lam = dp.lam, fs = dp.fs, nidx = dp.nidx;
    for (int j = 0; j < nv; ++j) {
        const size_t o = (size_t)s * nf + j;
        const int64_t i = idx[o];
        const double fx = F[i], fy = F[nf + i], fz = F[2 * nf + i];
        double dx = tx - fx, dy = ty - fy, dz = tz - fz;
        double Ttd = sqrt(dx * dx + dy * dy + dz * dz);
        double Jx = dx / Ttd, Jy = dy / Ttd, Jz = dz / Ttd;
        double Tth = acos(clamp1(-Jx * F[3 * nf + i] - Jy * F[4 * nf + i] - Jz * F[5 * nf + i]));
        double TarTh = acos(clamp1(-Jx * tnx - Jy * tny - Jz * tnz));
        double Tph = atan2(Jx * F[6 * nf + i] + Jy * F[7 * nf + i] + Jz * F[8 * nf + i],
                           Jx * F[9 * nf + i] + Jy * F[10 * nf + i] + Jz * F[11 * nf + i]);
        double expo = 0.0, tot = 0.0;
        for (int64_t k = 0; k < np; ++k) {
            double box[6] = {PR[np + k], PR[2 * np + k], PR[3 * np + k],
                             PR[4 * np + k], PR[5 * np + k], PR[6 * np + k]};
            double ad = d_prism_dist(fx, fy, fz, Jx, Jy, Jz, box, Ttd);
            tot += ad;
            expo += PR[k] * ad;
        }
        expo += dp.alpha2 * (Ttd - tot);
        double att = exp(-4 * expo);
        double cT = cos(Tth);
        double rough = exp(-4 * ((dp.ks * cT) * (dp.ks * cT)));
        double fEI = att, fEO = att;
        if (dp.specular) {
            // compRefrEnergyIn / compRefrEnergyOut facet reradiation
            // (geometry_kernels.cu:527-537, 563-570)
            fEI *= d_facet_rerad(Rth[o] - Tth, Iph[o] - Tph, lam, fs);
            double RrTh = d_snells(RP_PI_F - Tth, dp.eps2, dp.eps1);
            fEO *= d_facet_rerad(RrTh, Tph - Iph[o], lam, fs);
        }
        fEI = fEI * frc[o] * rough;
        fEO = fEO * frc[o] * rough;
        const double itd = Itd[o];
        if (ttype != 0) {
            double Gd = d_facet_G(TarTh, Tph, lam, fs);
            double Gt = d_facet_G(Tth, Tph, lam, fs);
            double Pin = d_friis(d_friis(dp.P, grefr, Gi[o], lam, itd), Gt, Gd, lam, Ttd);
            double Pout = d_friis(d_friis(1.0, grefr, Gi[o], lam, itd), Gt, Gd, lam, Ttd);
            if (!dp.lossless) { Pin *= fEI; Pout *= fEO; }
            double rngt = itd + Ttd * nidx;
            double x = (rngt - rst) / dp.dr;
            if (x > -1.0 && x < (double)nr) {
                long b = (long)x;
                double w = x - (double)b;
                double sn, cs;
                sincos(-(2.0 * RP_PI_F / lam) * rngt, &sn, &cs);
                double a = sqrt(Pin * nidx);
                C64 v{a * cs, a * sn};
                sincos(-(2.0 * RP_PI_F / lam) * (rngt - lam / 2.0), &sn, &cs);
                double a2 = sqrt(Pout * nidx);
                C64 u{a2 * cs, a2 * sn};
                pt[b] = cadd(pt[b], cscale(v, 1.0 - w));
                ps[b] = cadd(ps[b], cscale(u, 1.0 - w));
                if (b + 1 < nr) {
                    pt[b + 1] = cadd(pt[b + 1], cscale(v, w));
                    ps[b + 1] = cadd(ps[b + 1], cscale(u, w));
                }
            }
        } else if (dp.cmode == 2) {
            // refrRadarSignal's per-facet amplitude and range: rerad of the
            // facet-frame angle Tth and c / c2 (radar_kernels.cu:232-245)
            double rr = d_rerad(dp.rerad_funct, Tth) * fEI * fEO;
            double fSR = itd + Ttd;
            rr *= d_radar_eq(dp.P, grefr, fs, lam, fSR, (double)nv);
            PD[((size_t)s * tstride + q) * nf + j] = make_double2(rr, (fSR - Ttd) + Ttd * dp.c_over_c2);
        } else {
            double rr = d_rerad(dp.rerad_funct, TarTh) * fEI * fEO;
            double fSR = itd + Ttd;
            rr *= d_radar_eq(dp.P, grefr, fs, lam, fSR, (double)nv);
            double rngt = (fSR - Ttd) + Ttd * dp.c1_over_c2;
            double x = (rngt - rst) / dp.dr;
            if (x > -1.0 && x < (double)nr) {
                long b = (long)x;
                double sn, cs;
                sincos((4.0 * RP_PI_F / lam) * rngt, &sn, &cs);
                ps[b] = cadd(ps[b], C64{rr * cs, rr * sn});
            }
        }
    }
}

// Range compression per target: Ptarg = linconv(PTtarg, chirp2); the
// target's contribution = convolveComplex(Psour, Ptarg) (sim.cu:872, 912);
// ttype 0: linconv(phasor trace, chirp2) (sim.cu:963).  Result -> PT row.
// CT: the chirp spectrum of the target legs (chirp2; chirp1 in specular
// mode, which never regenerates it, sim.cu:851-856); CR, pR: the wrapped
// chirp of circular mode.
__global__ void k_conv64(const int* __restrict__ ntl, int64_t tstride, int nb,
                         const double* __restrict__ TG, int64_t nt, const int* __restrict__ tlist,
                         C64* __restrict__ PT, const C64* __restrict__ PS, const C64* __restrict__ C2,
                         PlanV<double> p2, PlanV<double> pN, int crop_K, int crop_all, int nr,
                         C64* __restrict__ scratch, size_t slot, int cmode, const C64* __restrict__ CR,
                         PlanV<double> pR) {
    C64* base = scratch + (size_t)blockIdx.x * slot;
    const int M = max(1 << p2.log2M, 1 << pN.log2M);
    C64* x = base;
    C64* wa = x + M;
    C64* wb = wa + M;
    C64* A = wb + M;
    C64* B = A + M;
    C64* ptarg = B + M;
    const int64_t items = (int64_t)nb * tstride;
    for (int64_t it = blockIdx.x; it < items; it += gridDim.x) {
        const int s = (int)(it / tstride);
        const int q = (int)(it % tstride);
        if (q >= ntl[s]) continue;
        const int64_t ti = tlist[(size_t)s * tstride + q];
        const int ttype = (int)TG[6 * nt + ti];
        C64* pt = PT + ((size_t)s * tstride + q) * nr;
        const C64* ps = PS + ((size_t)s * tstride + q) * nr;
        if (ttype != 0) {
            conv_linear_block<double>(pt, C2, p2, nr, x, wa, wb, ptarg, 1.0);
            conv_complex_block<double>(ps, ptarg, pN, nr, crop_K, crop_all, A, B, wa, wb, pt, 1.0);
        } else if (cmode == 0) {
            conv_linear_block<double>(ps, C2, p2, nr, x, wa, wb, pt, 1.0);
        } else if (cmode == 1) {
            conv_circular_block<double>(ps, CR, pR, nr, x, wa, wb, pt);       // sim.cu:959
        }
    }
}

// Surface: fixed point -> complex, disable_surface, linconv with chirp1
// (sim.cu:777-797).  One block per trace.
// mode: 0 non-specular (disable_surface applies), 1 specular linear (it does
// not, sim.cu:740-772), 2 zero (specular circular: the reference's surface
// convolution is commented out, sim.cu:765-767).
__global__ void k_surf_conv64(const long long* __restrict__ acc, const int* __restrict__ nill,
                              const unsigned long long* __restrict__ vmax, int disable, int nr,
                              const C64* __restrict__ C1, PlanV<double> p2,
                              C64* __restrict__ refl, C64* __restrict__ scratch, size_t slot, int mode) {
    const int s = blockIdx.x;
    if (mode == 2) {
        for (int i = threadIdx.x; i < nr; i += blockDim.x) refl[(size_t)s * nr + i] = C64{0.0, 0.0};
        return;
    }
    if (mode == 1) disable = 0;
    C64* base = scratch + (size_t)s * slot;
    const int M = 1 << p2.log2M;
    C64* x = base;
    C64* wa = x + M;
    C64* wb = wa + M;
    C64* in = wb + M;
    const int n = nill[s];
    double vm = __longlong_as_double((long long)vmax[s]);
    double inv = (n > 0 && vm > 0) ? (2.0 * (double)n * vm) / ldexp(1.0, RP_FIX_BITS) : 0.0;
    const long long* a = acc + (size_t)s * nr * 2;
    for (int i = threadIdx.x; i < nr; i += blockDim.x)
        in[i] = disable ? C64{0.0, 0.0} : C64{(double)a[2 * i] * inv, (double)a[2 * i + 1] * inv};
    __syncthreads();
    conv_linear_block<double>(in, C1, p2, nr, x, wa, wb, refl + (size_t)s * nr, 1.0);
}

// reflRadarSignal (radar_kernels.cu:58-160): per (trace, bin) the sum over the
// illuminated facets (facet order) of fRe sinc((rst + ir dr - Itd)/res)
// e^{+j 4 pi_F Itd / lam}.  Specular mode without convolution.
__global__ void k_direct_refl64(const int* __restrict__ nill, const double* __restrict__ Itd,
                                const double* __restrict__ fre, int64_t nf, const double* __restrict__ traces,
                                DevParams dp, C64* __restrict__ refl) {
    const int s = blockIdx.y;
    const int ir = blockIdx.x * blockDim.x + threadIdx.x;
    if (ir >= dp.nr) return;
    const TraceRow t = load_trace(traces, s);
    const double r = t.rst + ir * dp.dr;
    const int n = nill[s];
    C64 acc{0.0, 0.0};
    for (int j = 0; j < n; ++j) {
        const size_t o = (size_t)s * nf + j;
        const double d = Itd[o];
        double sn, cs;
        sincos((4.0 * RP_PI_F / dp.lam) * d, &sn, &cs);
        const double a = d_sinc((r - d) / dp.rng_res) * fre[o];
        acc.x += a * cs;
        acc.y += a * sn;
    }
    refl[(size_t)s * dp.nr + ir] = acc;
}

// refrRadarSignal (radar_kernels.cu:201-300): per (trace, target, bin) the sum
// over facets of rr sinc((rst + ir dr - rngt)/res) e^{+j 4 pi_F rngt / lam}
// from the (rr, rngt) pairs k_pairs64 left in PD.  Result: the target's row of Z.
__global__ void k_direct_refr64(const int* __restrict__ nill, const int* __restrict__ ntl, int64_t tstride,
                                int64_t nf, const double2* __restrict__ PD, const double* __restrict__ traces,
                                DevParams dp, C64* __restrict__ Z) {
    const int s = blockIdx.z;
    const int ir = blockIdx.x * blockDim.x + threadIdx.x;
    if (ir >= dp.nr) return;
    const TraceRow t = load_trace(traces, s);
    const double r = t.rst + ir * dp.dr;
    const int n = nill[s];
    for (int q = blockIdx.y; q < ntl[s]; q += gridDim.y) {
        const double2* pd = PD + ((size_t)s * tstride + q) * nf;
        C64 acc{0.0, 0.0};
        for (int j = 0; j < n; ++j) {
            const double2 v = pd[j];
            double sn, cs;
            sincos((4.0 * RP_PI_F / dp.lam) * v.y, &sn, &cs);
            const double a = d_sinc((r - v.y) / dp.rng_res) * v.x;
            acc.x += a * cs;
            acc.y += a * sn;
        }
        Z[((size_t)s * tstride + q) * dp.nr + ir] = acc;
    }
}

// sig = refl + sum_q refr_q in target order (sim.cu:980, 989).
__global__ void k_sum64(const int* __restrict__ nill, const int* __restrict__ ntl, int64_t tstride,
                        const C64* __restrict__ refl, const C64* __restrict__ Z, int nr,
                        void* __restrict__ out, int out64, int s0) {
    const int s = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nr) return;
    C64 v{0.0, 0.0};
    if (nill[s] > 0) {
        v = refl[(size_t)s * nr + i];
        const int n = ntl[s];
        const C64* z = Z + (size_t)s * tstride * nr + i;
        for (int q = 0; q < n; ++q) v = cadd(v, z[(size_t)q * nr]);
    }
    const size_t o = (size_t)(s0 + s) * nr + i;
    if (out64) reinterpret_cast<C64*>(out)[o] = v;
    else reinterpret_cast<float2*>(out)[o] = make_float2((float)v.x, (float)v.y);
}

// ---------------------------------------------------------------- plan ----
struct PlainLayout {
    int nb;            // traces in this batch
    int64_t tstride;   // max in-aperture targets per trace (upper bound)
    int slots;         // conv CTAs
    size_t slot;       // complex values per conv slot
    size_t surf_slot;
};

template <class A>
void plain_take(A& a, const rp_scene* sc, const PlainLayout& L) {
    const int64_t nf = std::max<int64_t>(sc->nf, 1), nt = std::max<int64_t>(sc->nt, 1);
    const int nr = sc->nr;
    const int tiles = (int)((std::max(nf, nt) + RP_TILE - 1) / RP_TILE);
    a.template take<uint8_t>((size_t)L.nb * nf);          // facet flags
    a.template take<int>((size_t)L.nb * tiles);            // tile counts
    a.template take<int>(L.nb);                            // nill
    a.template take<int>(L.nb);                            // ntl
    a.template take<unsigned long long>(L.nb);             // vmax
    a.template take<int>((size_t)L.nb * nf);               // idx
    a.template take<double>((size_t)L.nb * nf);            // Itd
    a.template take<double>((size_t)L.nb * nf);            // Gi
    a.template take<double>((size_t)L.nb * nf);            // fRfrC
    a.template take<double>((size_t)L.nb * nf);            // surface x
    a.template take<C64>((size_t)L.nb * nf);               // surface v
    a.template take<uint8_t>((size_t)L.nb * nt);           // target flags
    a.template take<int>((size_t)L.nb * nt);               // tlist
    a.template take<C64>((size_t)L.nb * L.tstride * nr);   // PT / Z
    a.template take<C64>((size_t)L.nb * L.tstride * nr);   // PS
    a.template take<long long>((size_t)L.nb * nr * 2);     // surface fixed point
    a.template take<C64>((size_t)L.nb * nr);               // refl
    a.template take<C64>((size_t)L.slots * L.slot);        // conv scratch
    a.template take<C64>((size_t)L.nb * L.surf_slot);      // surface conv scratch
    a.template take<double>((size_t)L.nb * nf);            // Rth
    a.template take<double>((size_t)L.nb * nf);            // Iph
    a.template take<double>((size_t)L.nb * nf);            // fRe
    if (sc->dp.cmode == 2) a.template take<double2>((size_t)L.nb * L.tstride * nf);   // (rr, rngt) per pair
}

PlainLayout plain_layout(const rp_scene* sc, int nb, int64_t tstride) {
    PlainLayout L;
    L.nb = nb;
    L.tstride = std::max<int64_t>(tstride, 1);
    const int M = std::max(sc->plan2.M(), sc->planN.M());
    L.slot = (size_t)5 * M + sc->nr;
    L.surf_slot = (size_t)3 * sc->plan2.M() + sc->nr;
    L.slots = std::max(1, 2 * sc->sm_count);
    return L;
}

const size_t kPlainBudget = (size_t)24 << 30;

// Upper bound of in-aperture targets per trace (host, FP64, aperture widened
// by 1e-9 rad so the device's exact count never exceeds it).
std::vector<int> host_target_bounds(const rp_scene* sc, const std::vector<double>& tr, int64_t ns,
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

size_t rp_plain_scratch(const rp_scene* sc, int64_t ns) {
    PlainLayout L = plain_layout(sc, (int)std::max<int64_t>(1, std::min<int64_t>(ns, 1)), sc->nt);
    ArenaPlan a;
    plain_take(a, sc, L);
    return a.off;
}

int rp_plain_run(rp_scene* sc, rp_workspace* ws, const double* d_traces, int64_t ns, void* d_out, int out64,
                 int64_t* h_counts, cudaStream_t st) {
    const int64_t nf = sc->nf, nt = sc->nt, np = sc->np;
    const int nr = sc->nr;
    if (sc->planN.pow2) { rp_set_error("internal: N = 2 nr - 1 is a power of two"); return RP_ERR_INTERNAL; }
    // host copies of the trace table and targets for the target bounds
    std::vector<double> tr(9 * ns), tg(7 * nt);
    RP_CUDA(cudaMemcpyAsync(tr.data(), d_traces, sizeof(double) * 9 * ns, cudaMemcpyDeviceToHost, st));
    if (nt) RP_CUDA(cudaMemcpyAsync(tg.data(), sc->d_targets, sizeof(double) * 7 * nt, cudaMemcpyDeviceToHost, st));
    RP_CUDA(cudaStreamSynchronize(st));
    std::vector<int> ub = host_target_bounds(sc, tr, ns, tg);
    PlanV<double> p2 = plan_view64(sc->plan2), pN = plan_view64(sc->planN);
    const size_t esz = out64 ? 16 : 8;
    for (int64_t s0 = 0; s0 < ns;) {
        // batch size from the memory budget
        int nb = 0;
        int64_t tmax = 0;
        for (;;) {
            if (s0 + nb >= ns) break;
            int64_t t2 = std::max<int64_t>(tmax, ub[s0 + nb]);
            PlainLayout L = plain_layout(sc, nb + 1, t2);
            ArenaPlan a;
            plain_take(a, sc, L);
            if (nb > 0 && a.off > kPlainBudget) break;
            tmax = t2;
            ++nb;
            if (nb >= 64) break;
        }
        PlainLayout L = plain_layout(sc, nb, tmax);
        ArenaPlan plan;
        plain_take(plan, sc, L);
        int rc = ws->arena.reserve(plan.off);
        if (rc) return rc;
        Arena& a = ws->arena;
        a.reset();
        const int64_t nfa = std::max<int64_t>(nf, 1), nta = std::max<int64_t>(nt, 1);
        const int tiles = (int)((std::max(nfa, nta) + RP_TILE - 1) / RP_TILE);
        uint8_t* fflags = a.take<uint8_t>((size_t)nb * nfa);
        int* tcnt = a.take<int>((size_t)nb * tiles);
        int* d_nill = a.take<int>(nb);
        int* d_ntl = a.take<int>(nb);
        unsigned long long* vmax = a.take<unsigned long long>(nb);
        int* idx = a.take<int>((size_t)nb * nfa);
        double* Itd = a.take<double>((size_t)nb * nfa);
        double* Gi = a.take<double>((size_t)nb * nfa);
        double* frc = a.take<double>((size_t)nb * nfa);
        double* sxv = a.take<double>((size_t)nb * nfa);
        C64* sv = a.take<C64>((size_t)nb * nfa);
        uint8_t* tflags = a.take<uint8_t>((size_t)nb * nta);
        int* tlist = a.take<int>((size_t)nb * nta);
        C64* PT = a.take<C64>((size_t)nb * L.tstride * nr);
        C64* PS = a.take<C64>((size_t)nb * L.tstride * nr);
        long long* acc = a.take<long long>((size_t)nb * nr * 2);
        C64* refl = a.take<C64>((size_t)nb * nr);
        C64* cscr = a.take<C64>((size_t)L.slots * L.slot);
        C64* sscr = a.take<C64>((size_t)nb * L.surf_slot);
        double* Rth = a.take<double>((size_t)nb * nfa);
        double* Iph = a.take<double>((size_t)nb * nfa);
        double* fre = a.take<double>((size_t)nb * nfa);
        double2* PD = (sc->dp.cmode == 2) ? a.take<double2>((size_t)nb * L.tstride * nfa) : nullptr;
        const DevParams& dp = sc->dp;
        const double* trb = d_traces + 9 * s0;

        g_timer.mark(0, st);
        RP_CUDA(cudaMemsetAsync(vmax, 0, sizeof(unsigned long long) * nb, st));
        RP_CUDA(cudaMemsetAsync(acc, 0, sizeof(long long) * nb * nr * 2, st));
        RP_CUDA(cudaMemsetAsync(PT, 0, sizeof(C64) * nb * L.tstride * nr, st));
        RP_CUDA(cudaMemsetAsync(PS, 0, sizeof(C64) * nb * L.tstride * nr, st));
        // facets: cull + compaction (geometry_kernels.cu:75-204)
        if (nf > 0) {
            k_cull_count<<<dim3((unsigned)((nf + RP_TILE - 1) / RP_TILE), nb), RP_TILE_THREADS, 0, st>>>(
                sc->d_facets, nf, trb, sc->dp.ap_rad, fflags, tcnt,
                reinterpret_cast<const double4*>(sc->d_tiles_file));
            RP_LAUNCHED();
            compact_flags(fflags, nf, nb, tcnt, d_nill, idx, nfa, true, st);
        } else {
            RP_CUDA(cudaMemsetAsync(d_nill, 0, sizeof(int) * nb, st));
        }
        // targets: aperture test + compaction (sim.cu:808-826)
        if (nt > 0) {
            k_target_flags<<<dim3((unsigned)((nt + 255) / 256), nb), 256, 0, st>>>(
                sc->d_targets, nt, trb, sc->dp.ap_rad, tflags);
            RP_LAUNCHED();
            compact_flags(tflags, nt, nb, tcnt, d_ntl, tlist, L.tstride, false, st);
        } else {
            RP_CUDA(cudaMemsetAsync(d_ntl, 0, sizeof(int) * nb, st));
        }
        if (nf > 0) {
            k_incident64<<<dim3((unsigned)((nf + 255) / 256), nb), 256, 0, st>>>(
                sc->d_facets, nf, idx, d_nill, trb, sc->dp, Itd, Gi, frc, sxv, sv, vmax, Rth, Iph, fre);
            RP_LAUNCHED();
            if (!dp.specular || dp.cmode == 0) {
                k_surf_fix64<<<dim3((unsigned)((nf + 255) / 256), nb), 256, 0, st>>>(
                    nfa, d_nill, sxv, sv, vmax, nr, acc, dp.specular);
                RP_LAUNCHED();
            }
        }
        g_timer.mark(1, st);
        if (nt > 0 && nf > 0 && tmax > 0) {
            k_pairs64<<<dim3((unsigned)((L.tstride + 63) / 64), nb), 64, 0, st>>>(
                sc->d_facets, nfa, idx, d_nill, sc->d_targets, nt, tlist, d_ntl, L.tstride,
                sc->d_prisms, np, trb, sc->dp, Itd, Gi, frc, PT, PS, Rth, Iph, PD);
            RP_LAUNCHED();
            ++g_timer.pair_launches;
            g_timer.mark(2, st);
            if (dp.cmode == 2) {
                k_direct_refr64<<<dim3((unsigned)((nr + 127) / 128), (unsigned)std::min<int64_t>(L.tstride, 65535), nb),
                                  128, 0, st>>>(
                    d_nill, d_ntl, L.tstride, nfa, PD, trb, dp, PT);
            } else {
                const C64* CT = (const C64*)(dp.specular ? sc->d_C1_64 : sc->d_C2_64);
                k_conv64<<<L.slots, 256, 0, st>>>(d_ntl, L.tstride, nb, sc->d_targets, nt, tlist, PT, PS,
                                                 CT, p2, pN, sc->crop_K, sc->crop_all, nr, cscr, L.slot,
                                                 dp.cmode, (const C64*)sc->d_CR_64,
                                                 dp.cmode == 1 ? plan_view64(sc->planR) : p2);
            }
            RP_LAUNCHED();
        }
        if (!(nt > 0 && nf > 0 && tmax > 0)) g_timer.mark(2, st);
        g_timer.mark(3, st);
        if (dp.specular && dp.cmode == 2) {
            k_direct_refl64<<<dim3((unsigned)((nr + 127) / 128), nb), 128, 0, st>>>(d_nill, Itd, fre, nfa, trb,
                                                                                  dp, refl);
        } else {
            const int smode = !dp.specular ? 0 : (dp.cmode == 0 ? 1 : 2);
            k_surf_conv64<<<nb, 256, 0, st>>>(acc, d_nill, vmax, sc->dp.disable_surface, nr,
                                             (const C64*)sc->d_C1_64, p2, refl, sscr, L.surf_slot, smode);
        }
        RP_LAUNCHED();
        k_sum64<<<dim3((nr + 255) / 256, nb), 256, 0, st>>>(d_nill, d_ntl, L.tstride, refl, PT, nr,
                                                           d_out, out64, (int)s0);
        RP_LAUNCHED();
        g_timer.mark(4, st);
        RP_CUDA(cudaGetLastError());
        if (g_timer.enabled) {
            RP_CUDA(cudaStreamSynchronize(st));
            g_timer.collect(0, 4);
        }
        if (h_counts) {
            std::vector<int> a1(nb), a2(nb);
            RP_CUDA(cudaMemcpyAsync(a1.data(), d_nill, sizeof(int) * nb, cudaMemcpyDeviceToHost, st));
            RP_CUDA(cudaMemcpyAsync(a2.data(), d_ntl, sizeof(int) * nb, cudaMemcpyDeviceToHost, st));
            RP_CUDA(cudaStreamSynchronize(st));
            for (int k = 0; k < nb; ++k) {
                h_counts[2 * (s0 + k)] = a1[k];
                h_counts[2 * (s0 + k) + 1] = a2[k];
            }
        } else if (s0 + nb < ns) {
            RP_CUDA(cudaStreamSynchronize(st));   // arena reuse across batches
        }
        (void)esz;
        s0 += nb;
    }
    return RP_OK;
}
