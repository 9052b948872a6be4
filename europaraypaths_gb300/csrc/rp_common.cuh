// rp_common.cuh -- per-trace stages shared by both forms: aperture culling of
// facets and targets, and the order-preserving (deterministic) compaction
// that replaces thrust::copy_if (geometry_kernels.cu:155-204).
#pragma once

#include "rp_math.cuh"

#define RP_TILE RP_CULL_TILE   // elements per compaction tile (and per culling sphere)
#define RP_TILE_THREADS 256

// Trace row: sx,sy,sz, snx,sny,snz, rst, grefl_lin, grefr_lin.
struct TraceRow {
    double sx, sy, sz, snx, sny, snz, rst, grefl, grefr;
};

__device__ __forceinline__ TraceRow load_trace(const double* tr, int s) {
    const double* r = tr + 9 * (size_t)s;
    return TraceRow{r[0], r[1], r[2], r[3], r[4], r[5], r[6], r[7], r[8]};
}

// Illumination test of compSourceInclination + cropByAperture
// (geometry_kernels.cu:75-100, 183-186): acos(-I . sn) < aperture, with the
// cosine clamped to [-1, 1].
__device__ __forceinline__ bool illuminated(double fx, double fy, double fz, const TraceRow& t,
                                            double ap_rad, double* dist) {
    double dx = fx - t.sx, dy = fy - t.sy, dz = fz - t.sz;
    double d = sqrt(dx * dx + dy * dy + dz * dz);
    *dist = d;
    double cs = clamp1((-dx / d) * t.snx + (-dy / d) * t.sny + (-dz / d) * t.snz);
    return acos(cs) < ap_rad;
}

// The same decision, cheaper: an FP32 cosine test decides every facet whose
// cosine is more than 1e-5 from cos(aperture) (the FP32 cosine is accurate to
// well under 1e-6 there, and acos is decreasing); facets inside that band
// take the exact FP64 test above.  *dist is set for illuminated facets only.
__device__ __forceinline__ bool illuminated_fast(double fx, double fy, double fz, const TraceRow& t,
                                                 double ap_rad, float ap_cos, double* dist) {
    const double dxd = fx - t.sx, dyd = fy - t.sy, dzd = fz - t.sz;
    const float dx = (float)dxd, dy = (float)dyd, dz = (float)dzd;
    const float c = -(dx * (float)t.snx + dy * (float)t.sny + dz * (float)t.snz) *
                    rsqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
    if (c < ap_cos - 1e-5f) return false;
    if (c > ap_cos + 1e-5f) {
        *dist = sqrt(dxd * dxd + dyd * dyd + dzd * dzd);
        return true;
    }
    return illuminated(fx, fy, fz, t, ap_rad, dist);
}

// Block-wide exclusive scan of one int per thread (blockDim.x <= 1024).
__device__ __forceinline__ int block_excl_scan(int v, int* total) {
    __shared__ int warp_sums[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int nw = (blockDim.x + 31) >> 5;
        int w = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    int base = wid ? warp_sums[wid - 1] : 0;
    if (total) *total = warp_sums[((blockDim.x + 31) >> 5) - 1];
    __syncthreads();
    return base + x - v;
}

// Whether every point of a tile's bounding sphere (c, r) lies outside the
// aperture cone of a trace: the angle of the centre from the look direction
// minus the sphere's angular radius exceeds the aperture by a margin far
// above FP64 rounding, so no facet that the exact test keeps is skipped.
__device__ __forceinline__ bool tile_outside(double4 sph, const TraceRow& t, double ap_rad) {
    const double vx = sph.x - t.sx, vy = sph.y - t.sy, vz = sph.z - t.sz;
    const double d = sqrt(vx * vx + vy * vy + vz * vz);
    if (!(d > sph.w)) return false;
    const double th = acos(clamp1(-(vx * t.snx + vy * t.sny + vz * t.snz) / d));
    return th - asin(sph.w / d) > ap_rad + 1e-9;
}

// Pass 1 of facet culling: the aperture flags and per-tile counts of
// illuminated facets.  grid (tiles, traces).  With tile spheres (one per
// RP_TILE facets of the store), a tile wholly outside the cone writes zero
// flags without reading its positions.
// pos: x,y,z SoA base (3 arrays of stride nf).
static __global__ void k_cull_count(const double* __restrict__ pos, int64_t nf,
                                    const double* __restrict__ traces, double ap_rad,
                                    uint8_t* __restrict__ flags, int* __restrict__ tile_cnt,
                                    const double4* __restrict__ tiles) {
    const int s = blockIdx.y;
    const TraceRow t = load_trace(traces, s);
    const float ap_cos = cosf((float)ap_rad);   // FP32: far inside the 1e-5 guard band
    const int64_t base = (int64_t)blockIdx.x * RP_TILE;
    // one thread decides for the block (FP64 transcendentals are slow on this GPU)
    __shared__ int s_skip;
    if (threadIdx.x == 0) s_skip = tiles != nullptr && tile_outside(tiles[blockIdx.x], t, ap_rad);
    __syncthreads();
    const bool skip = s_skip != 0;
    int cnt = 0;
    for (int k = threadIdx.x; k < RP_TILE; k += blockDim.x) {
        int64_t i = base + k;
        uint8_t f = 0;
        if (i < nf && !skip) {
            double d;       // unused here (the compiler drops its square root)
            f = illuminated_fast(pos[i], pos[nf + i], pos[2 * nf + i], t, ap_rad, ap_cos, &d) ? 1 : 0;
        }
        if (i < nf) flags[(size_t)s * nf + i] = f;
        cnt += f;
    }
    int tot;
    block_excl_scan(cnt, &tot);
    if (threadIdx.x == 0) tile_cnt[(size_t)s * gridDim.x + blockIdx.x] = tot;
}

// Pass 2: per trace, exclusive scan of the tile counts (one block per trace).
// A count above the list's capacity is cut to it and, with over != null,
// raises the flag (the host then reports an internal error).
static __global__ void k_scan_tiles(int* __restrict__ tile_cnt, int ntiles, int* __restrict__ total,
                                    int64_t cap, int* __restrict__ over) {
    const int s = blockIdx.x;
    int* c = tile_cnt + (size_t)s * ntiles;
    int carry = 0;
    for (int b0 = 0; b0 < ntiles; b0 += blockDim.x) {
        int i = b0 + threadIdx.x;
        int v = i < ntiles ? c[i] : 0;
        int tot;
        int ex = block_excl_scan(v, &tot);
        if (i < ntiles) c[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) {
        total[s] = (int)min((int64_t)carry, cap);
        if (over && (int64_t)carry > cap) atomicOr(over, 1);
    }
}

// Pass 3: scatter the original indices of flagged elements in order.
static __global__ void k_scatter(const uint8_t* __restrict__ flags, int64_t n,
                                 const int* __restrict__ tile_off, int ntiles,
                                 int* __restrict__ idx, int64_t idx_stride) {
    const int s = blockIdx.y;
    const int64_t base = (int64_t)blockIdx.x * RP_TILE;
    int pos = tile_off[(size_t)s * ntiles + blockIdx.x];
    const int per = RP_TILE / RP_TILE_THREADS;   // contiguous run per thread
    int f[RP_TILE / RP_TILE_THREADS];
    int cnt = 0;
    for (int k = 0; k < per; ++k) {
        int64_t i = base + (int64_t)threadIdx.x * per + k;
        f[k] = (i < n) ? flags[(size_t)s * n + i] : 0;
        cnt += f[k];
    }
    int ex = block_excl_scan(cnt, nullptr);
    int o = pos + ex;
    for (int k = 0; k < per; ++k) {
        int64_t i = base + (int64_t)threadIdx.x * per + k;
        if (f[k]) {
            if (o < idx_stride) idx[(size_t)s * idx_stride + o] = (int)i;
            ++o;
        }
    }
}

// Target aperture test of sim.cu:808-826 (acos(-sn . t_hat) > aperture -> skip).
static __global__ void k_target_flags(const double* __restrict__ tg, int64_t nt,
                                      const double* __restrict__ traces, double ap_rad,
                                      uint8_t* __restrict__ flags) {
    const int s = blockIdx.y;
    const TraceRow t = load_trace(traces, s);
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt) return;
    double vx = tg[i] - t.sx, vy = tg[nt + i] - t.sy, vz = tg[2 * nt + i] - t.sz;
    double m = sqrt(vx * vx + vy * vy + vz * vz);
    double th = acos(clamp1(-t.snx * vx / m - t.sny * vy / m - t.snz * vz / m));
    flags[(size_t)s * nt + i] = (th > ap_rad) ? 0 : 1;
}

static __global__ void k_fill_u64(unsigned long long* p, unsigned long long v, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

// Generic per-tile flag counter (targets).
static __global__ void k_count_flags(const uint8_t* __restrict__ flags, int64_t n,
                                     int* __restrict__ tile_cnt) {
    const int s = blockIdx.y;
    const int64_t base = (int64_t)blockIdx.x * RP_TILE;
    int cnt = 0;
    for (int k = threadIdx.x; k < RP_TILE; k += blockDim.x) {
        int64_t i = base + k;
        if (i < n) cnt += flags[(size_t)s * n + i];
    }
    int tot;
    block_excl_scan(cnt, &tot);
    if (threadIdx.x == 0) tile_cnt[(size_t)s * gridDim.x + blockIdx.x] = tot;
}

// Order-preserving compaction of per-trace flags (ns x n, uint8) into index
// lists idx (ns x stride); counts land in d_total.  When `counted` is set the
// per-tile counts are already in tile_cnt (the facet cull fuses them).
static inline void compact_flags(const uint8_t* flags, int64_t n, int ns, int* tile_cnt,
                                 int* d_total, int* idx, int64_t stride, bool counted,
                                 cudaStream_t st, int* over = nullptr) {
    const int nt = (int)((n + RP_TILE - 1) / RP_TILE);
    if (nt == 0 || ns == 0) {
        if (ns) cudaMemsetAsync(d_total, 0, sizeof(int) * ns, st);
        return;
    }
    if (!counted) {
        k_count_flags<<<dim3(nt, ns), RP_TILE_THREADS, 0, st>>>(flags, n, tile_cnt);
        RP_LAUNCHED();
    }
    k_scan_tiles<<<ns, 1024, 0, st>>>(tile_cnt, nt, d_total, stride, over);
    RP_LAUNCHED();
    k_scatter<<<dim3(nt, ns), RP_TILE_THREADS, 0, st>>>(flags, n, tile_cnt, nt, idx, stride);
    RP_LAUNCHED();
}
