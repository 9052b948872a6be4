"""NumPy FP64 restatement of the reference simulator's default path.

TEST INFRASTRUCTURE ONLY. The product (``europaraypaths_gb300``) never imports
this module: only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline leg may use it, and only as the checker.

It follows the reference line by line, vectorised over facets, for tiny scenes
(a few thousand facets, a handful of targets).  The C++ oracle
(``oracle/oracle.cpp``) is checked against it; both are checked against the
analytic known-answer formulas of the reference's validation scenes.

Modes covered: ``convolution=true, convolution_linear=true, specular=false``
(the default written by ``param_gen.gen_params``), with ``lossless``,
``disable_surface``, attenuation prisms and ``ttype`` 0/1 targets; and the
specular variants the reference defines: linear convolution (all targets),
no convolution and circular convolution (``ttype`` 0 targets only).

Reference citations are ``file:line`` inside the reference project.
"""
import numpy as np

PI_F = 3.14159265          # geometry_kernels.cu:45 / radar_kernels.cu:682 constant
PI_FRIIS = 3.14159         # geometry_kernels.cu:411, file_io.cu:196 constant


def sinc(x):
    """elementary_kernels.cu:50-53: sin(pi x)/(pi x), 1 for |x| < 1e-6."""
    x = np.asarray(x, dtype=np.float64)
    out = np.ones_like(x)
    m = np.abs(x) >= 1e-6
    out[m] = np.sin(np.pi * x[m]) / (np.pi * x[m])
    return out


def facet_G(th, ph, lam, fs):
    """radar_kernels.cu:658-677 (the sinc argument carries pi twice)."""
    piLlam = PI_F * fs / lam
    s1 = sinc(piLlam * np.sin(th) * np.cos(ph))
    s2 = sinc(piLlam * np.sin(th) * np.sin(ph))
    return (s1 * s2) ** 2 * (4 * PI_F * fs * fs) / (lam * lam)


def friis(P, Gt, Gr, lam, dist):
    """geometry_kernels.cu:410-412."""
    return (P * lam * lam * Gt * Gr) / ((4 * PI_FRIIS) ** 2 * dist * dist)


def radar_eq(P, G, fs, lam, dist, nfacets):
    """geometry_kernels.cu:384-393."""
    return nfacets * (P * G * G * fs ** 4) / ((4 * PI_FRIIS) ** 2 * dist ** 4)


def phasor(r, lam):
    """radar_kernels.cu:681-686: exp(-j 2 pi r / lam)."""
    return np.exp(-1j * (2.0 * PI_F / lam) * r)


def rerad_funct(funcnum, th1):
    """radar_kernels.cu:167-189 (case 3 multiplies by pi/180, as written)."""
    th1 = np.asarray(th1, dtype=np.float64)
    if funcnum == 0:
        return np.ones_like(th1)
    if funcnum == 1:
        return (th1 * (180 / PI_F) < 1).astype(np.float64)
    if funcnum == 2:
        return (th1 * (180 / PI_F) < 0.5).astype(np.float64)
    if funcnum == 3:
        return (th1 * (PI_F / 180) < 3).astype(np.float64)
    if funcnum == 4:
        sigma = PI_F / 180
        return np.exp(-0.5 * th1 ** 2 / (sigma * sigma))
    return np.ones_like(th1)


def facet_rerad(th, ph, lam, fs):
    """facetReradiation, geometry_kernels.cu:353-381."""
    s1 = sinc((fs / lam) * np.sin(th) * np.cos(ph))
    s2 = sinc((fs / lam) * np.sin(th) * np.sin(ph))
    return ((fs * fs / lam) * s1 * s2) ** 2


def snells(th, e1, e2):
    """snellsLaw, geometry_kernels.cu:490-501 (1e4 on total internal reflection)."""
    sR = np.sqrt(e1 / e2) * np.sin(th)
    return np.where(sR > 1.0, 1e4, np.arcsin(np.minimum(sR, 1.0)))


def single_bin_trace(nr, x, ph):
    """genReflPhasor/genRefrPhasor + genPhasorTrace: one truncated bin per
    facet, out-of-range facets dropped (radar_kernels.cu:314-451)."""
    b = np.trunc(x).astype(np.int64)
    bad = (b < 0) | (b >= nr)
    b[bad] = 0
    ph = np.where(bad, 0.0, ph)
    tr = np.zeros(nr, np.complex128)
    np.add.at(tr, b, ph)
    return tr


def direct_sum(nr, rst, dr, res, rng, amp, lam):
    """reflRadarSignal / refrRadarSignal: sum_f amp sinc((r - rng)/res) e^{j 4 pi rng / lam}
    over every bin r = rst + ir dr (radar_kernels.cu:58-160, 201-300)."""
    r = rst + np.arange(nr) * dr
    ph = np.exp(1j * (4.0 * PI_F / lam) * rng) * amp
    return (sinc((r[:, None] - rng[None, :]) / res) * ph[None, :]).sum(axis=1)


def conv_circular(trace, chirp, nr):
    """convolvePhasorChirp, radar_kernels.cu:516-552."""
    return np.fft.ifft(np.fft.fft(trace) * np.fft.fft(chirp.astype(np.complex128)))


def trunc_bin(x):
    """(short)x in the reference: truncation toward zero (radar_kernels.cu:736-737)."""
    b = np.trunc(x).astype(np.int64)
    return b, x - b


def chirp_padded(nr, dr, res):
    """genCenteredChirpPadded, radar_kernels.cu:489-503 (length 2 nr)."""
    i = np.arange(2 * nr)
    return sinc((i - nr // 2) * dr / res)


def conv_linear(trace, chirp, nr):
    """convolvePhasorChirpLinear, radar_kernels.cu:554-649."""
    n2 = 2 * nr
    a = np.zeros(n2, np.complex128)
    a[:nr] = trace
    y = np.fft.ifft(np.fft.fft(a) * np.fft.fft(chirp.astype(np.complex128)))
    # cuFFT inverse is unnormalised, then scaled by 1/(2 nr): same as numpy's ifft
    return y[nr // 2: nr // 2 + nr].copy()


def conv_complex(sig, ker, nr, smpl, B):
    """convolveComplex + cropSpectrum + takeEveryOtherComplex,
    elementary_kernels.cu:258-353 and :187-194 (length N = 2 nr - 1)."""
    N = 2 * nr - 1
    a = np.zeros(N, np.complex128)
    b = np.zeros(N, np.complex128)
    a[:nr] = sig
    b[:nr] = ker
    A = np.fft.fft(a)
    Bk = np.fft.fft(b)
    k = np.arange(N)
    freq = np.where(k <= N // 2, k * smpl / N, (k - N) * smpl / N)
    Bk[np.abs(freq) > B] = 0.0
    z = np.fft.ifft(A * Bk)
    return z[0:2 * nr:2][:nr].copy()


def bin_split_add(trace, nr, x, contrib):
    """Two-bin linear split used by surfacePT/accumulateTarget/radiateTarget
    (radar_kernels.cu:748-760).  bin+1 == nr is dropped (the reference writes
    one element past its buffer there)."""
    b, w = trunc_bin(x)
    ok = (b >= 0) & (b < nr)
    b, w, c = b[ok], w[ok], contrib[ok]
    np.add.at(trace, b, c * (1.0 - w))
    ok2 = b + 1 < nr
    np.add.at(trace, b[ok2] + 1, c[ok2] * w[ok2])


def prism_distance(o, d, box, t):
    """prismIntersectionDistance, geometry_kernels.cu:207-269 (vectorised)."""
    INF = 1e30
    tlo = np.full(o.shape[0], -INF)
    thi = np.full(o.shape[0], INF)
    miss = np.zeros(o.shape[0], bool)
    for ax in range(3):
        lo, hi = box[ax], box[ax + 3]
        par = np.abs(d[:, ax]) < 1e-12
        miss |= par & ((o[:, ax] < lo) | (o[:, ax] > hi))
        with np.errstate(divide="ignore", invalid="ignore"):
            t1 = (lo - o[:, ax]) / d[:, ax]
            t2 = (hi - o[:, ax]) / d[:, ax]
        a1 = np.where(par, -INF, np.minimum(t1, t2))
        a2 = np.where(par, INF, np.maximum(t1, t2))
        tlo = np.maximum(tlo, a1)
        thi = np.minimum(thi, a2)
    tlo = np.maximum(tlo, 0.0)
    thi = np.minimum(thi, t)
    out = np.where(tlo >= thi, 0.0, thi - tlo)
    out[miss] = 0.0
    return out


def _mix64(z):
    """SplitMix64's mixing function on uint64 arrays (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9e3779b97f4a7c15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xbf58476d1ce4e5b9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94d049bb133111eb)
        return z ^ (z >> np.uint64(31))


def incoherent_turns(seed, S, idx):
    """Incoherent mode's seeded surface phases in turns (the reference draws
    them from clock64(), radar_kernels.cu:689-711): SplitMix64 mixing over
    (seed, the bits of the source position S, the facets' input indices),
    the top 24 bits as k / 2^24."""
    bits = np.asarray(S, dtype=np.float64).view(np.uint64)
    key = _mix64(np.array([seed], dtype=np.uint64))
    for b in bits:
        key = _mix64(key ^ b)
    r = _mix64(key ^ np.asarray(idx, dtype=np.uint64))
    return (r >> np.uint64(40)).astype(np.float64) / 16777216.0


def simulate(p, facets, targets, traces, prisms=None):
    """Run the reference trace loop (sim.cu:615-1008) in FP64.

    p        dict of derived parameters (see ``derive``)
    facets   (N, 12) float64: x,y,z, nx,ny,nz, ux,uy,uz, vx,vy,vz
    targets  (T, 7)  float64: x,y,z, nx,ny,nz, ttype
    traces   (S, 9)  float64: sx,sy,sz, snx,sny,snz, rst, grefl_lin, grefr_lin
    prisms   (P, 7)  float64: alpha, xmin,ymin,zmin, xmax,ymax,zmax  (or None)

    Returns (S, nr) complex128 and the (S, 2) counts (N_ill, N_t in aperture).
    """
    nr, dr = p["nr"], p["dr"]
    lam, fs = p["lam"], p["fs"]
    ap = p["aperture"] * (np.pi / 180.0)
    out = np.zeros((traces.shape[0], nr), np.complex128)
    counts = np.zeros((traces.shape[0], 2), np.int64)
    F = facets
    chirp1 = chirp_padded(nr, dr, p["rng_res"])
    chirp2 = chirp_padded(nr, dr, 2 * p["rng_res"])
    spec = bool(p.get("specular", False))
    cmode = 2 if not p.get("convolution", True) else (0 if p.get("convolution_linear", True) else 1)
    chirpT = chirp1 if spec else chirp2            # specular never regenerates the chirp
    ii = np.arange(nr)
    chirpR = sinc(ii * dr / p["rng_res"]) + sinc((ii - nr) * dr / p["rng_res"])   # genChirp
    n_idx = np.sqrt(p["eps_2"])
    for s in range(traces.shape[0]):
        S = traces[s, 0:3]
        sn = traces[s, 3:6]
        rst = traces[s, 6]
        grefl = traces[s, 7]
        grefr = traces[s, 8]
        # compSourceInclination + cropByAperture (geometry_kernels.cu:75-204)
        d = F[:, 0:3] - S
        itd = np.sqrt(np.sum(d * d, axis=1))
        I = d / itd[:, None]
        cosv = np.clip(np.sum(-I * sn, axis=1), -1.0, 1.0)
        ill = np.arccos(cosv) < ap
        f = F[ill]
        nv = f.shape[0]
        counts[s, 0] = nv
        if nv == 0:
            continue
        # compIncidentRays (geometry_kernels.cu:103-140)
        d = f[:, 0:3] - S
        Itd = np.sqrt(np.sum(d * d, axis=1))
        I = d / Itd[:, None]
        Ith = np.arccos(np.clip(np.sum(-I * f[:, 3:6], axis=1), -1.0, 1.0))
        Iph = np.arctan2(np.sum(I * f[:, 6:9], axis=1), np.sum(I * f[:, 9:12], axis=1))
        # compRefractedRays / snellsLaw (geometry_kernels.cu:490-517)
        sR = np.sqrt(p["eps_1"] / p["eps_2"]) * np.sin(Ith)
        Rth = np.where(sR > 1.0, 1e4, np.arcsin(np.minimum(sR, 1.0)))
        # compReflectedEnergy, non-specular, H-pol (geometry_kernels.cu:426-487)
        cI, cR = np.cos(Ith), np.cos(Rth)
        rho = (p["nu_2"] * cI - p["nu_1"] * cR) / (p["nu_2"] * cI + p["nu_1"] * cR)
        fRfrC = 1.0 - rho * rho
        fRe = rho * rho
        if spec:
            fRe = facet_rerad(2 * Ith, -Iph, lam, fs) * radar_eq(p["P"], grefl, fs, lam, Itd, nv) * fRe
        fRfrC = np.where(Rth > 1e3, 0.0, fRfrC)
        atm = np.exp(-4.0 * p["alpha1"] * Itd)
        fRe = fRe * atm
        fRfrC = fRfrC * atm
        fRe = fRe * np.exp(-4 * (p["ks"] * cI) ** 2)
        # surfacePT (radar_kernels.cu:714-764)
        G = facet_G(Ith, Iph, lam, fs)
        Pf = friis(p["P"], grefr, G, lam, Itd)
        Ps = friis(Pf, G, grefr, lam, Itd)
        if not p["lossless"]:
            Ps = Ps * fRe
        if not spec:
            psurf = np.zeros(nr, np.complex128)
            if p.get("incoherent", False):      # randomPhasor (radar_kernels.cu:741-742), seeded
                ph = np.exp(2j * np.pi * incoherent_turns(p["incoherent_seed"], S, np.nonzero(ill)[0]))
            else:
                ph = phasor(2 * Itd, lam)
            bin_split_add(psurf, nr, (Itd - rst) / dr, ph * np.sqrt(Ps))
            if p["disable_surface"]:
                psurf[:] = 0.0
            refl = conv_linear(psurf, chirp1, nr)
        elif cmode == 0:
            tr = single_bin_trace(nr, (Itd - rst) / dr, np.exp(1j * (4.0 * PI_F / lam) * Itd) * fRe)
            refl = conv_linear(tr, chirp1, nr)
        elif cmode == 2:
            refl = direct_sum(nr, rst, dr, p["rng_res"], Itd, fRe, lam)
        else:
            refl = np.zeros(nr, np.complex128)
        # target loop (sim.cu:801-986)
        refr = np.zeros(nr, np.complex128)
        nt_in = 0
        for t in range(targets.shape[0]):
            T = targets[t, 0:3]
            tn = targets[t, 3:6]
            ttype = int(targets[t, 6])
            tv = T - S
            tv = tv / np.sqrt(np.sum(tv * tv))
            th = np.arccos(np.clip(np.sum(-sn * tv), -1.0, 1.0))
            if th > ap:
                continue
            nt_in += 1
            # compTargetRays (geometry_kernels.cu:272-350)
            dt = T - f[:, 0:3]
            Ttd = np.sqrt(np.sum(dt * dt, axis=1))
            J = dt / Ttd[:, None]
            Tth = np.arccos(np.clip(np.sum(-J * f[:, 3:6], axis=1), -1.0, 1.0))
            TarTh = np.arccos(np.clip(np.sum(-J * tn, axis=1), -1.0, 1.0))
            Tph = np.arctan2(np.sum(J * f[:, 6:9], axis=1), np.sum(J * f[:, 9:12], axis=1))
            expo = np.zeros(nv)
            tot = np.zeros(nv)
            if prisms is not None:
                for pr in prisms:
                    dist = prism_distance(f[:, 0:3], J, pr[1:7], Ttd)
                    tot += dist
                    expo += pr[0] * dist
            expo += p["alpha2"] * (Ttd - tot)
            att = np.exp(-4 * expo)
            rough_t = np.exp(-4 * (p["ks"] * np.cos(Tth)) ** 2)
            # compRefrEnergyIn / compRefrEnergyOut (geometry_kernels.cu:520-584)
            fEI = att.copy()
            fEO = att.copy()
            if spec:
                fEI = fEI * facet_rerad(Rth - Tth, Iph - Tph, lam, fs)
                fEO = fEO * facet_rerad(snells(PI_F - Tth, p["eps_2"], p["eps_1"]), Tph - Iph, lam, fs)
            fEI = fEI * fRfrC * rough_t
            fEO = fEO * fRfrC * rough_t
            fSR = Itd + Ttd
            if ttype != 0:
                # accumulateTarget (radar_kernels.cu:767-830)
                Gd = facet_G(TarTh, Tph, lam, fs)
                Gi = facet_G(Ith, Iph, lam, fs)
                Gt = facet_G(Tth, Tph, lam, fs)
                Pin = friis(friis(p["P"], grefr, Gi, lam, Itd), Gt, Gd, lam, Ttd)
                Pout = friis(friis(1.0, grefr, Gi, lam, Itd), Gt, Gd, lam, Ttd)
                if not p["lossless"]:
                    Pin = Pin * fEI
                    Pout = Pout * fEO
                rngt = Itd + Ttd * n_idx
                pt = np.zeros(nr, np.complex128)
                bin_split_add(pt, nr, (rngt - rst) / dr, phasor(rngt, lam) * np.sqrt(Pin * n_idx))
                ptarg = conv_linear(pt, chirpT, nr)
                # radiateTarget (radar_kernels.cu:834-892)
                ps = np.zeros(nr, np.complex128)
                bin_split_add(ps, nr, (rngt - rst) / dr,
                              phasor(rngt - lam / 2.0, lam) * np.sqrt(Pout * n_idx))
                refr += conv_complex(ps, ptarg, nr, p["smpl"], p["B"])
            elif cmode == 2:
                # refrRadarSignal: rerad of Tth, c / c2 (radar_kernels.cu:201-300)
                rr = rerad_funct(p["rerad_funct"], Tth) * fEI * fEO
                rr = rr * radar_eq(p["P"], grefr, fs, lam, fSR, nv)
                rngt = (fSR - Ttd) + Ttd * (p["c"] / p["c_2"])
                refr += direct_sum(nr, rst, dr, p["rng_res"], rngt, rr, lam)
            else:
                # genRefrPhasor + genPhasorTrace + linear conv (radar_kernels.cu:351-448)
                rr = rerad_funct(p["rerad_funct"], TarTh) * fEI * fEO
                rr = rr * radar_eq(p["P"], grefr, fs, lam, fSR, nv)
                rngt = (fSR - Ttd) + Ttd * (p["c_1"] / p["c_2"])
                ph = np.exp(1j * (4.0 * PI_F / lam) * rngt) * rr
                b = np.trunc((rngt - rst) / dr).astype(np.int64)
                bad = (b < 0) | (b >= nr)
                b[bad] = 0
                ph[bad] = 0.0
                tr = np.zeros(nr, np.complex128)
                np.add.at(tr, b, ph)
                refr += conv_linear(tr, chirpT, nr) if cmode == 0 else conv_circular(tr, chirpR, nr)
        counts[s, 1] = nt_in
        out[s] = refl + refr
    return out, counts


def derive(j):
    """Derived constants of parseSimulationParameters, file_io.cu:122-249.

    ``j`` is the JSON dict.  Everything is FP64 except ``nr``, which follows
    the reference's float expression exactly (file_io.cu:212) so that the
    range-bin count is identical.
    """
    c = 299792458.0
    nu0 = 376.7
    eps_0 = 8.85e-12
    f0 = float(j["frequency"])
    B = float(j["bandwidth"])
    lam = c / f0
    k = 2 * PI_F / lam
    p = dict(c=c, f0=f0, B=B, P=float(j["power"]), aperture=float(j["aperture"]),
             lam=lam, k=k, rng_res=c / B, fs=float(j["fs"]))
    p["Grefr_lin"] = 10 ** (float(j.get("subsurface_gain", 0.0)) / 10.0)
    p["Grefl_lin"] = 10 ** (float(j.get("surface_gain", 0.0)) / 10.0)
    p["rms_h"] = float(j["rms_height"])
    p["ks"] = k * p["rms_h"]
    for key in ("eps_1", "eps_2", "sig_1", "sig_2"):
        p[key] = float(j[key])
    p["c_1"] = c / np.sqrt(p["eps_1"])
    p["c_2"] = c / np.sqrt(p["eps_2"])
    p["nu_1"] = nu0 / np.sqrt(p["eps_1"])
    p["nu_2"] = nu0 / np.sqrt(p["eps_2"])

    def alpha(sig, eps):
        epp = sig / (2 * PI_FRIIS * f0 * eps_0)
        a = np.sqrt(1 + (epp / eps) ** 2) - 1
        a = np.sqrt(0.5 * eps * a)
        return a * 2 * PI_FRIIS / lam

    p["alpha1"] = alpha(p["sig_1"], p["eps_1"])
    p["alpha2"] = alpha(p["sig_2"], p["eps_2"])
    p["smpl"] = float(j["rx_sample_rate"])
    f32 = np.float32
    nr = int(f32(f32(j["rx_window_m"]) / f32(299792480.0)) * f32(p["smpl"]))
    p["nr"] = nr
    p["dr"] = float(j["rx_window_m"]) / nr
    p["rerad_funct"] = int(j.get("rerad_funct", 1))
    p["lossless"] = bool(j.get("lossless", False))
    p["incoherent"] = bool(j.get("incoherent", False))
    p["incoherent_seed"] = int(j.get("incoherent_seed", 1))
    p["disable_surface"] = bool(j.get("disable_surface", False))
    p["specular"] = bool(j.get("specular", False))
    p["convolution"] = bool(j.get("convolution", True))
    p["convolution_linear"] = bool(j.get("convolution_linear", True))
    return p


def prism_alpha(sig, p):
    """loadAttenPrismFile conductivity -> alpha (file_io.cu:502-505)."""
    eps_0 = 8.85e-12
    epp = sig / (2 * PI_FRIIS * p["f0"] * eps_0)
    a = np.sqrt(1 + (epp / p["eps_2"]) ** 2) - 1
    a = np.sqrt(0.5 * p["eps_2"] * a)
    return a * 2 * PI_FRIIS / p["lam"]
