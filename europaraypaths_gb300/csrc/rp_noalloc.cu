// rp_noalloc.cu -- surface-only radargram columns computed without any device
// allocation: the per-call scratch lives in a fixed array inside the library.
//
// Who needs this: callers whose device memory is fixed when they start and
// that may not allocate afterwards -- e.g. a processing loop that runs inside
// a device-memory budget owned by someone else (a host application whose own
// allocator holds the GPU's memory, or a long-running service that must not
// grow or fragment its footprint after initialisation).  They create the
// scene once at set-up (rp_scene_create allocates then) and afterwards call
// rp_surface_noalloc, which calls no cudaMalloc, cudaFree or other
// allocating routine.
//
// One kernel block per trace does the whole surface leg: the aperture test,
// the per-facet incident leg (compIncidentRays, snellsLaw,
// compReflectedEnergy and surfacePT; geometry_kernels.cu:103-140, 426-517,
// radar_kernels.cu:714-764), fixed-point binning, and the linear chirp
// convolution (convolvePhasorChirpLinear, radar_kernels.cu:554-649).
// Precision: the incident leg runs in FP64 here, angles included, where the
// resident fast form's facet kernel takes its angles in FP32; the phasors
// are rounded to FP32 for binning and the convolution is the fast form's
// FP32 transform.  The columns therefore agree with rp_simulate_device's
// fast form to about 1e-7 relative L2 (the test holds 1e-6) and with the
// FP64 oracle to the same order (the test holds 1e-5), not bit for bit.
//
// Cost: the block walks the scene's 1024-facet culling tiles; a tile whose
// bounding sphere lies wholly outside the trace's aperture cone is skipped
// without reading its facets, so each trace evaluates the facets of the
// tiles that touch its footprint, twice (once for the count and the
// fixed-point scale, once to bin).
#include <cuda_runtime.h>

#include "rp_common.cuh"
#include "rp_conv.cuh"

// Limits of the fixed scratch array.
#define RP_NOALLOC_MAX_TRACES 16
#define RP_NOALLOC_MAX_BINS 4096
#define RP_NOALLOC_SCRATCH_BYTES (16u << 20)

// The scratch every call shares: per trace, 2 nr int64 fixed-point bins, nr
// complex inputs and three FFT buffers.  Its contents persist between calls;
// the kernel clears the bins it uses before accumulating.  Calls that overlap
// on the GPU (different streams, or different host threads without ordering)
// race on this array and must not be issued.
static __device__ __align__(256) unsigned char g_noalloc_scratch[RP_NOALLOC_SCRATCH_BYTES];

namespace {

using C32 = Cx<float>;

size_t noalloc_slot_bytes(int nr, int M) {
    size_t b = (size_t)2 * nr * sizeof(long long);       // fixed-point bins
    b = (b + 255) & ~size_t(255);
    b += (size_t)nr * sizeof(C32);                        // compression input
    b = (b + 255) & ~size_t(255);
    b += (size_t)3 * M * sizeof(C32);                     // x, wa, wb
    return (b + 255) & ~size_t(255);
}

struct NoallocArgs {
    const int64_t* order;   // sorted facet position -> input index (incoherent phases)
    const double* F;      // sorted facet store, FP64 SoA [12][nf]
    int64_t nf;
    const double4* tiles;   // bounding sphere per RP_CULL_TILE sorted facets (may be null)
    const double* traces;
    DevParams dp;
    const C32* C1;
    PlanV<float> p2;
    unsigned char* scratch;
    size_t slot;
    float2* out;
};

__device__ __forceinline__ void surface_leg(const NoallocArgs& A, const TraceRow& t, int64_t i, bool* ok,
                                            float* x, C32* v, double* amp_o) {
    const double* F = A.F;
    const int64_t nf = A.nf;
    const DevParams& dp = A.dp;
    double d;
    *ok = illuminated(F[i], F[nf + i], F[2 * nf + i], t, dp.ap_rad, &d);
    if (!*ok) return;
    double dx = F[i] - t.sx, dy = F[nf + i] - t.sy, dz = F[2 * nf + i] - t.sz;
    d = sqrt(dx * dx + dy * dy + dz * dz);
    double Ix = dx / d, Iy = dy / d, Iz = dz / d;
    double th = acos(clamp1(-Ix * F[3 * nf + i] - Iy * F[4 * nf + i] - Iz * F[5 * nf + i]));
    double ph = atan2(Ix * F[6 * nf + i] + Iy * F[7 * nf + i] + Iz * F[8 * nf + i],
                      Ix * F[9 * nf + i] + Iy * F[10 * nf + i] + Iz * F[11 * nf + i]);
    double sR = sqrt(dp.eps1 / dp.eps2) * sin(th);
    double rth = sR > 1.0 ? 1e4 : asin(sR);
    double cI = cos(th), cR = cos(rth);
    double rho = (dp.nu2 * cI - dp.nu1 * cR) / (dp.nu2 * cI + dp.nu1 * cR);
    double fre = rho * rho;
    fre *= exp(-4.0 * dp.alpha1 * d);
    fre *= exp(-4 * ((dp.ks * cI) * (dp.ks * cI)));
    double G = d_facet_G(th, ph, dp.lam, dp.fs);
    double Pf = d_friis(dp.P, t.grefr, G, dp.lam, d);
    double Ps = d_friis(Pf, G, t.grefr, dp.lam, d);
    if (!dp.lossless) Ps *= fre;
    double amp = sqrt(Ps);
    double sn, cs;
    if (dp.incoherent) {        // the seeded phases of incoherent mode (rp_incoherent_turns)
        sincospi(2.0 * rp_incoherent_turns(dp.inc_seed, t.sx, t.sy, t.sz, A.order[i]), &sn, &cs);
    } else {
        double tt = 2.0 * d * dp.turn;
        double ft = tt - floor(tt);
        sincospi(-2.0 * ft, &sn, &cs);
    }
    *x = (float)((d - t.rst) / dp.dr);
    *v = C32{(float)(amp * cs), (float)(amp * sn)};
    *amp_o = amp;
}

// Whether tile tb of the sorted store may hold illuminated facets (one
// thread tests the tile's sphere; the answer is block-uniform).
__device__ __forceinline__ bool tile_live(const NoallocArgs& A, const TraceRow& t, int64_t tb, int* s_live) {
    if (threadIdx.x == 0) s_live[0] = (A.tiles == nullptr) || !tile_outside(A.tiles[tb], t, A.dp.ap_rad);
    __syncthreads();
    const bool live = s_live[0] != 0;
    __syncthreads();   // everyone has read the flag before thread 0 rewrites it
    return live;
}

__global__ void __launch_bounds__(256) k_surface_noalloc(NoallocArgs A) {
    __shared__ double sh_max[32];
    __shared__ int sh_cnt[32];
    __shared__ int s_live[1];
    const int s = blockIdx.x;
    const int nr = A.dp.nr;
    const TraceRow t = load_trace(A.traces, s);
    unsigned char* base = A.scratch + (size_t)s * A.slot;
    long long* acc = reinterpret_cast<long long*>(base);
    size_t off = (((size_t)2 * nr * sizeof(long long)) + 255) & ~size_t(255);
    C32* in = reinterpret_cast<C32*>(base + off);
    off = (off + (size_t)nr * sizeof(C32) + 255) & ~size_t(255);
    const int M = 1 << A.p2.log2M;
    C32* x = reinterpret_cast<C32*>(base + off);
    C32* wa = x + M;
    C32* wb = wa + M;
    for (int i = threadIdx.x; i < 2 * nr; i += blockDim.x) acc[i] = 0;   // bins start at zero
    // pass 1: illuminated count and the largest amplitude (the fixed-point scale)
    const int64_t ntiles = (A.nf + RP_CULL_TILE - 1) / RP_CULL_TILE;
    int cnt = 0;
    double vm = 0.0;
    for (int64_t tb = 0; tb < ntiles; ++tb) {
        if (!tile_live(A, t, tb, s_live)) continue;
        const int64_t end = min(A.nf, (tb + 1) * (int64_t)RP_CULL_TILE);
        for (int64_t i = tb * RP_CULL_TILE + threadIdx.x; i < end; i += blockDim.x) {
            bool ok; float xx; C32 v; double amp;
            surface_leg(A, t, i, &ok, &xx, &v, &amp);
            if (ok) { ++cnt; vm = fmax(vm, amp); }
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        vm = fmax(vm, __shfl_xor_sync(0xffffffffu, vm, o));
    }
    if (lane == 0) { sh_cnt[wid] = cnt; sh_max[wid] = vm; }
    __syncthreads();
    int n = 0;
    vm = 0.0;
    for (int w = 0; w < nw; ++w) { n += sh_cnt[w]; vm = fmax(vm, sh_max[w]); }
    float2* orow = A.out + (size_t)s * nr;
    if (n == 0) {   // no illuminated facet: a zero column (the reference skips the file)
        for (int i = threadIdx.x; i < nr; i += blockDim.x) orow[i] = make_float2(0.f, 0.f);
        return;
    }
    // pass 2: fixed-point binning (order-independent integer sums)
    if (vm > 0) {
        const double scale = ldexp(1.0, RP_FIX_BITS) / (2.0 * (double)n * vm);
        for (int64_t tb = 0; tb < ntiles; ++tb) {
            if (!tile_live(A, t, tb, s_live)) continue;
            const int64_t end = min(A.nf, (tb + 1) * (int64_t)RP_CULL_TILE);
            for (int64_t i = tb * RP_CULL_TILE + threadIdx.x; i < end; i += blockDim.x) {
                bool ok; float xf; C32 v; double amp;
                surface_leg(A, t, i, &ok, &xf, &v, &amp);
                if (!ok) continue;
                double xx = xf;
                if (!(xx > -1.0) || xx >= (double)nr) continue;
                long b = (long)xx;
                double w = xx - (double)b;
                fix_add(acc + 2 * b, (double)v.x * (1.0 - w), scale);
                fix_add(acc + 2 * b + 1, (double)v.y * (1.0 - w), scale);
                if (b + 1 < nr) {
                    fix_add(acc + 2 * (b + 1), (double)v.x * w, scale);
                    fix_add(acc + 2 * (b + 1) + 1, (double)v.y * w, scale);
                }
            }
        }
    }
    __syncthreads();
    const double inv = (vm > 0) ? (2.0 * (double)n * vm) / ldexp(1.0, RP_FIX_BITS) : 0.0;
    for (int i = threadIdx.x; i < nr; i += blockDim.x)
        in[i] = A.dp.disable_surface ? C32{0.f, 0.f}
                                     : C32{(float)((double)acc[2 * i] * inv), (float)((double)acc[2 * i + 1] * inv)};
    __syncthreads();
    conv_linear_block<float>(in, A.C1, A.p2, nr, x, wa, wb, reinterpret_cast<C32*>(orow), 1.0f);
}

}  // namespace

extern "C" int rp_surface_noalloc(const rp_scene* s, const double* d_traces, int64_t ns, void* d_out,
                                  void* stream) {
    if (!s || ns < 0 || (ns > 0 && (!d_traces || !d_out))) {
        rp_set_error("rp_surface_noalloc: bad argument");
        return RP_ERR_ARG;
    }
    if (s->dp.specular) {
        rp_set_error("rp_surface_noalloc: the default (non-specular) mode only; specular scenes use "
                     "rp_simulate_device");
        return RP_ERR_UNSUPPORTED;
    }
    if (ns == 0) return RP_OK;
    const int nr = s->nr;
    if (ns > RP_NOALLOC_MAX_TRACES || nr > RP_NOALLOC_MAX_BINS) {
        rp_set_error("rp_surface_noalloc: %lld traces x %d bins exceed the fixed scratch limits "
                     "(at most %d traces and %d range bins per call)",
                     (long long)ns, nr, RP_NOALLOC_MAX_TRACES, RP_NOALLOC_MAX_BINS);
        return RP_ERR_BUDGET;
    }
    const size_t slot = noalloc_slot_bytes(nr, s->plan2.M());
    if (slot * (size_t)ns > RP_NOALLOC_SCRATCH_BYTES) {
        rp_set_error("rp_surface_noalloc: %lld traces need %zu bytes of scratch, more than the fixed "
                     "%u bytes", (long long)ns, slot * (size_t)ns, RP_NOALLOC_SCRATCH_BYTES);
        return RP_ERR_BUDGET;
    }
    if (s->device < 0 || s->device >= 64) { rp_set_error("rp_surface_noalloc: device ordinal"); return RP_ERR_ARG; }
    RP_CUDA(cudaSetDevice(s->device));
    // The array's device address in the current context, looked up on every
    // call (no allocation; the first call in a context also loads the
    // library's module): a cached address would go stale if the context were
    // reset and re-created.
    void* ptr = nullptr;
    {
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return rp_cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    }
    NoallocArgs A;
    A.F = s->d_sorted;
    A.order = s->d_order;
    A.nf = s->nf;
    A.tiles = reinterpret_cast<const double4*>(s->d_tiles_sorted);
    A.traces = d_traces;
    A.dp = s->dp;
    A.C1 = reinterpret_cast<const C32*>(s->d_C1_32);
    A.p2 = plan_view32(s->plan2);
    A.scratch = static_cast<unsigned char*>(ptr);
    A.slot = slot;
    A.out = static_cast<float2*>(d_out);
    cudaStream_t st = stream ? (cudaStream_t)stream : s->own_stream;
    k_surface_noalloc<<<(unsigned)ns, 256, 0, st>>>(A);
    RP_CUDA(cudaGetLastError());
    return RP_OK;
}
