// rp_internal.h -- shared host/device definitions of libraypath.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/raypath.h"

// Constants exactly as the reference spells them.
#define RP_PI_F 3.14159265      // geometry_kernels.cu:45, radar_kernels.cu:682
#define RP_PI_FRIIS 3.14159     // geometry_kernels.cu:411, file_io.cu:196
#define RP_PI 3.14159265358979323846

// Output flag OR'ed into `form`: write complex128 instead of complex64.
#define RP_OUT_COMPLEX128 0x100

// Fixed-point scale headroom for deterministic integer accumulation.
#define RP_FIX_BITS 60

// Polls of an mbarrier before a pair kernel's wait for a staged chunk gives
// up (RP_ERR_TIMEOUT), and the short limit of the stalled-copy test mode.
// Elements of the range compression's shared-memory transform buffer (128
// KiB): mode 2 runs its sub-blocks, or at 2nr = 2 RP_CONV_CHUNK its two
// halves, in it (rp_convs.cu); the chirp spectrum of such a scene is stored
// in the halves' order.
#define RP_CONV_CHUNK 16384
#define RP_SPIN_LIMIT (1 << 22)
#define RP_SPIN_LIMIT_TEST 4096

void rp_set_error(const char* fmt, ...);
#define RP_CULL_TILE 1024   // facets per compaction tile and per culling sphere

int rp_cuda_fail(cudaError_t e, const char* what);
// Raise fn's dynamic shared-memory limit to at least bytes (never lowers it).
int rp_allow_dyn_smem(const void* fn, size_t bytes);

#define RP_CUDA(call)                                                    \
    do {                                                                 \
        cudaError_t _e = (call);                                         \
        if (_e != cudaSuccess) return rp_cuda_fail(_e, #call);           \
    } while (0)

// Device-side copy of the constants every kernel needs (FP64).
struct DevParams {
    double lam, fs, P, nidx, eps1, eps2, nu1, nu2, alpha1, alpha2, ks, c1_over_c2;
    double dr, smpl, B, rng_res, ap_rad, ap_cos;
    double inv_dr, sqrt_eps12;   // 1 / dr, sqrt(eps1 / eps2) (fast-form setup)
    unsigned long long inc_seed; // incoherent mode: the phase hash's seed
    int incoherent;              // incoherent mode: surface phasors from rp_incoherent_turns
    double turn;   // phase turns per metre of range: pi_F / (pi lam), so that
                   // exp(-j (2 pi_F / lam) r) = exp(-j 2 pi r turn) (radar_kernels.cu:682)
    int nr, lossless, disable_surface, rerad_funct;
    int ortho;           // facet frames orthonormal: records carry a.u, a.v instead of n
    int specular;        // specular mode (geometry_kernels.cu:434-446, 527-537, 563-570)
    int cmode;           // 0 linear convolution, 1 circular, 2 none (sim.cu:733-986)
    double c_over_c2;    // c / c_2 of refrRadarSignal's range (radar_kernels.cu:245)
};

// Grow-only device arena for per-call scratch.
struct Arena {
    void* ptr = nullptr;
    size_t cap = 0;
    size_t off = 0;
    int reserve(size_t bytes);          // make sure cap >= bytes (frees old)
    void reset() { off = 0; }
    template <class T>
    T* take(size_t n) {
        size_t a = (off + 255) & ~size_t(255);
        off = a + n * sizeof(T);
        return reinterpret_cast<T*>(static_cast<char*>(ptr) + a);
    }
    void release();
};

// Bytes a take<T>(n) sequence needs, for sizing an Arena.
struct ArenaPlan {
    size_t off = 0;
    template <class T>
    void take(size_t n) { off = ((off + 255) & ~size_t(255)) + n * sizeof(T); }
};

// A DFT of length n on the device: a radix-2 FFT when n is a power of two,
// else Bluestein's chirp-z transform through a power-of-two length M.
struct DftPlan {
    int n = 0;
    int pow2 = 0;          // n is a power of two
    int log2M = 0;         // log2 of the FFT length actually run (n or M)
    double* tw64 = nullptr;   // e^{-2 pi i k / M}, k < M/2
    double* bw64 = nullptr;   // Bluestein w_k = e^{-i pi k^2 / n}, k < n
    double* bW64 = nullptr;   // FFT_M of the conjugate chirp
    float* tw32 = nullptr;
    float* bw32 = nullptr;
    float* bW32 = nullptr;
    int M() const { return 1 << log2M; }
};

// Per-call scratch of one stream of work: scenes are shared and read-only
// during a simulation; everything a call writes lives here.
struct rp_workspace {
    int device = 0;
    Arena arena;     // setup buffers
    Arena arena2;    // pair-stage buffers, sized once the target-window width is known
    // auxiliary streams: the segments of a multi-segment wave run their
    // (small, independent) setup and tail kernels concurrently on these,
    // forked from and joined back into the caller's stream by events
    static const int kAux = 4;
    cudaStream_t aux[kAux] = {};
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_join[kAux] = {};
    bool aux_ready = false;
    int ensure_aux();                                   // create them once (on the current device)
    void fork(cudaStream_t st);                         // aux streams wait for st
    void join(cudaStream_t st);                         // st waits for the aux streams
    // ---- graph capture (rp_graph_*).  graph_mode 1: an eager call planned
    // from plan_traces (host [ns][9]; a batch: plan_jobs, one per job) with
    // target windows from host bounds;
    // 2: the same call under stream capture -- no host syncs or readbacks,
    // no tuning probes, job tables staged in the pinned arena, and each
    // segment's flags and counts copied into it (graph_rb) for
    // rp_graph_check after the replay.
    int graph_mode = 0;
    const double* plan_traces = nullptr;
    std::vector<const double*> plan_jobs;
    char* pin = nullptr;            // pinned host arena (graph mode 2)
    size_t pin_cap = 0, pin_off = 0;
    struct Readback { const int* misc; const int* cnt; int nb; int64_t s0; };   // s0: first trace, over all jobs
    std::vector<Readback> graph_rb;
    void* pin_take(size_t bytes) {                      // nullptr when full
        const size_t a = (pin_off + 255) & ~size_t(255);
        if (!pin || a + bytes > pin_cap) return nullptr;
        pin_off = a + bytes;
        return pin + a;
    }
};

struct rp_scene {
    rp_params p;
    DevParams dp;
    int device = 0;
    int64_t nf = 0, nt = 0, np = 0;
    int nr = 0;
    // ---- plain store: original facet order, FP64 SoA [12][nf]
    double* d_facets = nullptr;
    // ---- targets FP64 SoA [7][nt], prisms FP64 SoA [7][np]
    double* d_targets = nullptr;
    double* d_prisms = nullptr;
    std::vector<double> h_targets;       // host copy of the targets (aperture bounds)
    int any_ttype0 = 0;
    // the fast form's copy of the targets, ttype-1 targets first (stable), so
    // each trace's ordered in-aperture list is both kinds' lists in turn;
    // the same pointer as d_targets when every target is ttype 1
    double* d_targets_fast = nullptr;
    int64_t nt1 = 0;                     // ttype-1 targets (the first nt1 of d_targets_fast)
    // ---- fast store: spatially sorted facets
    int64_t* d_order = nullptr;          // sorted position -> original index
    double* d_tiles_sorted = nullptr;    // per RP_CULL_TILE sorted facets: bounding sphere (x, y, z, r)
    std::vector<double> h_tiles_sorted;  // the same on the host (per-trace facet bounds)
    double* d_tiles_file = nullptr;      // the same for the input-order store
    double* d_sorted = nullptr;          // FP64 SoA [12][nf] in sorted order
    // ---- per-scene spectral tables
    DftPlan plan2;                       // length 2 nr (linear chirp convolution)
    DftPlan planN;                       // length N = 2 nr - 1 (convolveComplex)
    DftPlan planR;                       // length nr (circular convolution mode only)
    double* d_CR_64 = nullptr;           // DFT_nr of genChirp's wrapped chirp (circular mode)
    float* d_CR_32 = nullptr;
    double* d_C1_64 = nullptr;           // DFT_2nr of the surface chirp (complex)
    double* d_C2_64 = nullptr;           // DFT_2nr of the target chirp (complex)
    float* d_C1_32 = nullptr;
    float* d_C2_32 = nullptr;
    int crop_K = 0;                      // kept spectrum half-width on the N grid
    int crop_all = 0;                    // crop keeps every bin
    // shared-memory compression tables (nr a power of two): FP32, spectra in
    // the digit-reversed order of the in-place DIF stages (rp_fft.cuh)
    int smem_conv = 0;                   // tables present
    int mS = 0, log2mS = 0;              // M = 4 nr
    float* d_C2S = nullptr;              // DIF_2nr(target chirp)
    float* d_HS = nullptr;               // DIF_M(crop kernel h) / M
    // ---- tuning
    int ortho = 0;                       // every facet frame (n, u, v) orthonormal to 1e-5
    int pair_variant = 0;                // 0 auto (polynomial sinc where accurate), 1 special-function sinc
    int pair_cfg = 3;                    // pair-kernel configuration without tuning, and the tuner's
                                         // default (3: 4 facet pairs per step x 2 blocks per SM)
    int spin_limit = RP_SPIN_LIMIT;      // polls of a pair kernel's chunk wait before it gives up
    int stall_copies = 0;                // test mode (RP_TEST_STALL_COPIES): the pair kernels issue
                                         // no bulk copy, so their first wait runs out (short limit)
    // ---- the scene's own workspace (rp_simulate / rp_simulate_device)
    rp_workspace ws;
    cudaStream_t own_stream = nullptr;
    int sm_count = 0;
    size_t store_bytes = 0;
};

// Per-thread launch counter (rp_last_launch_count).
extern thread_local int64_t g_launches;
#define RP_LAUNCHED() (++g_launches)

// Per-thread stage timing with CUDA events on the launching stream
// (rp_set_timing / rp_last_timing).  Stages: 0 cull + per-facet setup,
// 1 pair kernel, 2 per-target range compression, 3 surface + final sum.
#define RP_NSTAGE 4
struct StageTimer {
    int enabled = 0;
    double ms[RP_NSTAGE] = {0, 0, 0, 0};
    int64_t pair_launches = 0;
    cudaEvent_t ev[RP_NSTAGE + 1] = {};
    int have_events = 0;
    void reset() {
        for (int i = 0; i < RP_NSTAGE; ++i) ms[i] = 0;
        pair_launches = 0;
    }
    void mark(int i, cudaStream_t st);          // record boundary event i
    void collect(int first, int last);          // add elapsed of stages first..last-1 (after sync)
};
extern thread_local StageTimer g_timer;

// Entry points of the two forms (rp_plain.cu, rp_fast.cu).
int rp_plain_run(rp_scene* s, rp_workspace* ws, const double* d_traces, int64_t ns, void* d_out,
                 int out64, int64_t* h_counts, cudaStream_t st);
int rp_fast_run(rp_scene* s, rp_workspace* ws, const double* d_traces, int64_t ns, void* d_out,
                int out64, int64_t* h_counts, cudaStream_t st);
int rp_fast_batch(const rp_job* jobs, int njobs, rp_workspace* ws, cudaStream_t st);
size_t rp_plain_scratch(const rp_scene* s, int64_t ns);
size_t rp_fast_scratch(const rp_scene* s, int64_t ns);
