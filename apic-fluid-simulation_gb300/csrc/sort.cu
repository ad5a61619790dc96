// sort.cu — Morton keys, stable LSD radix sort, particle permutation.
//
// Restates Apic::update_spatial_lookup (src/apic.rs:1043-1111): key = Morton
// code of the particle's clamped cell (:1049-1064), sort of (key, val = slot)
// pairs (:1066, rdst radix_sort_unstable over 4 x 8-bit levels, :220-227), then
// a gather of the nine particle fields by `val` with the tail lanes of the last
// chunk zero-filled (:1068-1104).  The reference leaves the order of equal keys
// to rdst; this sort is stable (equal keys keep ascending `val`), which is the
// order the oracle defines.
//
// Per pass over one 8-bit digit: a histogram kernel (warp match + shared
// counters), a device-wide exclusive scan of the digit-major histogram, and a
// scatter kernel that ranks keys stably inside its tile with __match_any_sync
// (per-warp running counters, then a per-digit prefix over warps).  Only the
// digits below the bit length of the largest possible key are sorted: higher
// digits are zero for every key, so their passes are identities.
#include <cuda_runtime.h>

#include "apic_device.cuh"
#include "apic_internal.h"

namespace apic {

namespace {

constexpr int kItems = kSortTile / kSortThreads;  // 8 keys per thread
constexpr int kScanBlock = 1024;                  // elements per scan block

__global__ void k_morton_keys(const PartPtrs* __restrict__ pp, uint32_t n, float dx, float max_x, float max_y,
                              uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    pdl_wait();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float gx = pp->f[PX][i] / dx, gy = pp->f[PY][i] / dx;  // Vec2x8 / f32x8: per-component division
    uint32_t cx = uint32_t(trunc_x86(fmin_x86(fmax_x86(gx, 0.0f), max_x)));
    uint32_t cy = uint32_t(trunc_x86(fmin_x86(fmax_x86(gy, 0.0f), max_y)));
    keys[i] = morton(cx, cy);
    vals[i] = i;
}

// Per-tile digit histogram, written digit-major: hist[d * nblocks + b].
__global__ void __launch_bounds__(kSortThreads) k_sort_hist(const uint32_t* __restrict__ keys, uint32_t n,
                                                             int shift, uint32_t* __restrict__ hist) {
    pdl_wait();
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t base = blockIdx.x * kSortTile + warp * (kSortTile / kSortThreads * 32);
    for (int r = 0; r < kItems; ++r) {
        uint32_t i = base + r * 32 + lane;
        uint32_t d = i < n ? (keys[i] >> shift) & 0xFFu : 256u;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        if (d < 256u && (peers & ((1u << lane) - 1u)) == 0) atomicAdd(&h[d], uint32_t(__popc(peers)));
    }
    __syncthreads();
    hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one tile; offs = exclusive scan of hist.
__global__ void __launch_bounds__(kSortThreads) k_sort_scatter(const uint32_t* __restrict__ keys,
                                                                const uint32_t* __restrict__ vals, uint32_t n,
                                                                int shift, const uint32_t* __restrict__ offs,
                                                                uint32_t* __restrict__ okeys,
                                                                uint32_t* __restrict__ ovals) {
    pdl_wait();
    __shared__ uint32_t wh[kSortThreads / 32][256];
    __shared__ uint32_t boff[256];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int w = 0; w < kSortThreads / 32; ++w) wh[w][threadIdx.x] = 0;
    boff[threadIdx.x] = offs[threadIdx.x * gridDim.x + blockIdx.x];
    __syncthreads();
    uint32_t base = blockIdx.x * kSortTile + warp * (kItems * 32);
    uint32_t k[kItems], v[kItems], rk[kItems];
    uint32_t lt = (1u << lane) - 1u;
    for (int r = 0; r < kItems; ++r) {
        uint32_t i = base + r * 32 + lane;
        bool ok = i < n;
        k[r] = ok ? keys[i] : 0u;
        v[r] = ok ? vals[i] : 0u;
        uint32_t d = ok ? (k[r] >> shift) & 0xFFu : 256u;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t before = ok ? wh[warp][d] : 0u;
        __syncwarp();
        if (ok && (peers & lt) == 0) wh[warp][d] = before + uint32_t(__popc(peers));
        __syncwarp();
        rk[r] = before + uint32_t(__popc(peers & lt));
    }
    __syncthreads();
    {
        uint32_t run = 0;
        for (int w = 0; w < kSortThreads / 32; ++w) {
            uint32_t c = wh[w][threadIdx.x];
            wh[w][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
    for (int r = 0; r < kItems; ++r) {
        uint32_t i = base + r * 32 + lane;
        if (i >= n) continue;
        uint32_t d = (k[r] >> shift) & 0xFFu;
        uint32_t pos = boff[d] + wh[warp][d] + rk[r];
        okeys[pos] = k[r];
        ovals[pos] = v[r];
    }
}

// ---- device-wide exclusive scan of u32 (three kernels, no inter-block waits)
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t sw[32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sw[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < int(blockDim.x / 32) ? sw[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        sw[lane] = s;
    }
    __syncthreads();
    uint32_t pre = warp > 0 ? sw[warp - 1] : 0u;
    *total = sw[blockDim.x / 32 - 1];
    __syncthreads();
    return pre + x - v;
}

__global__ void __launch_bounds__(256) k_scan_reduce(const uint32_t* __restrict__ in, uint32_t n,
                                                     uint32_t* __restrict__ bsum) {
    pdl_wait();
    uint32_t b0 = blockIdx.x * kScanBlock;
    uint32_t s = 0;
    for (int k = 0; k < kScanBlock / 256; ++k) {
        uint32_t i = b0 + k * 256 + threadIdx.x;
        if (i < n) s += in[i];
    }
    __shared__ uint32_t red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) bsum[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(1024) k_scan_blocksums(uint32_t* __restrict__ bsum, uint32_t nb) {
    pdl_wait();
    uint32_t carry = 0;
    for (uint32_t c = 0; c < nb; c += 1024) {
        uint32_t i = c + threadIdx.x;
        uint32_t v = i < nb ? bsum[i] : 0u;
        uint32_t tot;
        uint32_t ex = block_exclusive_scan(v, &tot);
        if (i < nb) bsum[i] = carry + ex;
        carry += tot;
    }
}

__global__ void __launch_bounds__(256) k_scan_down(uint32_t* __restrict__ data, uint32_t n,
                                                   const uint32_t* __restrict__ bsum) {
    pdl_wait();
    uint32_t b0 = blockIdx.x * kScanBlock;
    uint32_t carry = bsum[blockIdx.x];
    for (int k = 0; k < kScanBlock / 256; ++k) {
        uint32_t i = b0 + k * 256 + threadIdx.x;
        uint32_t v = i < n ? data[i] : 0u;
        uint32_t tot;
        uint32_t ex = block_exclusive_scan(v, &tot);
        if (i < n) data[i] = carry + ex;
        carry += tot;
    }
}

}  // namespace

cudaError_t exclusive_scan_u32(uint32_t* data, uint32_t n, uint32_t* tmp, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    uint32_t nb = div_up(n, kScanBlock);
    launch(st != nullptr, k_scan_reduce, nb, 256, 0, st, data, n, tmp);
    launch(st != nullptr, k_scan_blocksums, 1, 1024, 0, st, tmp, nb);
    launch(st != nullptr, k_scan_down, nb, 256, 0, st, data, n, tmp);
    return cudaGetLastError();
}

static int key_bits(const Scene& s) {
    uint32_t mx = s.W ? s.W - 1 : 0, my = s.H ? s.H - 1 : 0;
    // Morton order is monotone in x and y, so the largest key is that of the far corner.
    uint32_t ex = mx & 0xFFFFu, ey = my & 0xFFFFu;
    auto expand = [](uint32_t v) {
        v = (v | (v << 8)) & 0x00FF00FFu;
        v = (v | (v << 4)) & 0x0F0F0F0Fu;
        v = (v | (v << 2)) & 0x33333333u;
        v = (v | (v << 1)) & 0x55555555u;
        return v;
    };
    uint32_t k = expand(ex) | (expand(ey) << 1);
    int b = 0;
    while (b < 32 && (k >> b)) ++b;
    return b;
}

cudaError_t launch_sort(Scene& s) {
    if (s.n == 0) return cudaSuccess;
    float max_x = float(s.W > 0 ? s.W - 1 : 0), max_y = float(s.H > 0 ? s.H - 1 : 0);
    launch(s.use_pdl, k_morton_keys, div_up(s.n, 256), 256, 0, s.stream, s.pp, s.n, s.dx, max_x, max_y, s.keys, s.vals);
    uint32_t nb = div_up(s.n, kSortTile);
    int bits = key_bits(s);
    uint32_t* k_in = s.keys;
    uint32_t* v_in = s.vals;
    uint32_t* k_out = s.keys_alt;
    uint32_t* v_out = s.vals_alt;
    for (int shift = 0; shift < bits; shift += 8) {
        launch(s.use_pdl, k_sort_hist, nb, kSortThreads, 0, s.stream, k_in, s.n, shift, s.sort_hist);
        cudaError_t e = exclusive_scan_u32(s.sort_hist, 256u * nb, s.sort_scan_tmp, s.stream);
        if (e != cudaSuccess) return e;
        launch(s.use_pdl, k_sort_scatter, nb, kSortThreads, 0, s.stream, k_in, v_in, s.n, shift, s.sort_hist, k_out, v_out);
        std::swap(k_in, k_out);
        std::swap(v_in, v_out);
    }
    if (k_in != s.keys) {  // keep the sorted pairs in keys/vals
        cudaMemcpyAsync(s.keys, k_in, sizeof(uint32_t) * s.n, cudaMemcpyDeviceToDevice, s.stream);
        cudaMemcpyAsync(s.vals, v_in, sizeof(uint32_t) * s.n, cudaMemcpyDeviceToDevice, s.stream);
    }
    return launch_permute(s);
}

// Stable LSD sort of (keys, vals)[0..n) over the low `bits` key bits, with all
// intermediate storage supplied by the caller: keys_alt/vals_alt (n words
// each), hist (256 * ceil(n / 2048) words) and scan_tmp (ceil(hist / 1024)
// words).  The sorted pairs end in keys/vals.
cudaError_t radix_sort_pairs_in(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, uint32_t* hist,
                                uint32_t* scan_tmp, uint32_t n, int bits, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    uint32_t nb = div_up(n, kSortTile);
    uint32_t* k_in = keys;
    uint32_t* v_in = vals;
    uint32_t* k_out = keys_alt;
    uint32_t* v_out = vals_alt;
    for (int shift = 0; shift < bits; shift += 8) {
        launch(st != nullptr, k_sort_hist, nb, kSortThreads, 0, st, k_in, n, shift, hist);
        cudaError_t e = exclusive_scan_u32(hist, 256u * nb, scan_tmp, st);
        if (e != cudaSuccess) return e;
        launch(st != nullptr, k_sort_scatter, nb, kSortThreads, 0, st, k_in, v_in, n, shift, hist, k_out, v_out);
        std::swap(k_in, k_out);
        std::swap(v_in, v_out);
    }
    if (k_in != keys) {
        cudaMemcpyAsync(keys, k_in, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(vals, v_in, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st);
    }
    return cudaGetLastError();
}

// Bit length of the largest Morton key of a width x height grid.
int morton_key_bits(uint32_t width, uint32_t height) {
    Scene probe;
    probe.W = width;
    probe.H = height;
    return key_bits(probe);
}

}  // namespace apic
