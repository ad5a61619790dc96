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
// Per pass over one digit of up to 10 bits: a histogram kernel (warp match +
// shared counters), a device-wide exclusive scan of the digit-major
// histogram, and a scatter kernel that ranks keys stably inside its tile with
// __match_any_sync and writes them through a shared-memory stage.  Only the
// bits below the bit length of the largest possible key are sorted: higher
// bits are zero for every key, so their passes would be identities.  The
// digit width is chosen per sort for the fewest passes (20-bit keys of a
// 1024^2 grid: two 10-bit passes), and the sorted pairs stay in the buffer
// the last pass wrote.
#include <cuda_runtime.h>

#include "apic_device.cuh"
#include "apic_internal.h"

namespace apic {

namespace {

constexpr int kItems = kSortTile / kSortThreads;  // 8 keys per thread
constexpr uint32_t kMaxBuckets = 1u << kMaxDigitBits;
constexpr int kScanBlock = 1024;                  // elements per scan block

// Four particles per thread with 16-byte loads and stores: the particle
// arrays and the pair buffers hold npad (a multiple of 8) lanes, so lanes
// n .. npad-1 get keys too, which the sort of n pairs never reads.
__global__ void __launch_bounds__(256) k_morton_keys(const PartPtrs* __restrict__ pp, uint32_t n, float dx, float max_x,
                                                     float max_y, uint32_t* __restrict__ keys,
                                                     uint32_t* __restrict__ vals) {
    pdl_wait();
    const uint32_t i0 = 4u * (blockIdx.x * blockDim.x + threadIdx.x);
    if (i0 >= n) return;
    const float4 px = *reinterpret_cast<const float4*>(pp->f[PX] + i0);
    const float4 py = *reinterpret_cast<const float4*>(pp->f[PY] + i0);
    const float xs[4] = {px.x, px.y, px.z, px.w}, ys[4] = {py.x, py.y, py.z, py.w};
    uint32_t k[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float gx = xs[q] / dx, gy = ys[q] / dx;  // Vec2x8 / f32x8: per-component division
        const uint32_t cx = uint32_t(trunc_x86(fmin_x86(fmax_x86(gx, 0.0f), max_x)));
        const uint32_t cy = uint32_t(trunc_x86(fmin_x86(fmax_x86(gy, 0.0f), max_y)));
        k[q] = morton(cx, cy);
    }
    *reinterpret_cast<uint4*>(keys + i0) = make_uint4(k[0], k[1], k[2], k[3]);
    *reinterpret_cast<uint4*>(vals + i0) = make_uint4(i0, i0 + 1, i0 + 2, i0 + 3);
}

// Per-tile digit histogram of a `dbits`-bit digit (dbits <= kMaxDigitBits),
// written digit-major: hist[d * nblocks + b].
__global__ void __launch_bounds__(kSortThreads) k_sort_hist(const uint32_t* __restrict__ keys, uint32_t n,
                                                             int shift, int dbits, uint32_t* __restrict__ hist) {
    pdl_wait();
    __shared__ uint32_t h[kMaxBuckets];
    const uint32_t nbk = 1u << dbits, mask = nbk - 1u;
    for (uint32_t d = threadIdx.x; d < nbk; d += kSortThreads) h[d] = 0;
    __syncthreads();
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t base = blockIdx.x * kSortTile + warp * (kSortTile / kSortThreads * 32);
    for (int r = 0; r < kItems; ++r) {
        uint32_t i = base + r * 32 + lane;
        uint32_t d = i < n ? (keys[i] >> shift) & mask : kMaxBuckets;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        if (d < kMaxBuckets && (peers & ((1u << lane) - 1u)) == 0) atomicAdd(&h[d], uint32_t(__popc(peers)));
    }
    __syncthreads();
    for (uint32_t d = threadIdx.x; d < nbk; d += kSortThreads) hist[d * gridDim.x + blockIdx.x] = h[d];
}

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total);

// Stable scatter of one tile; offs = exclusive scan of hist.  Keys are ranked
// inside the tile with __match_any_sync (per-warp running counters, then a
// prefix over warps and over digits), staged in shared memory in the tile's
// sorted order, and written out so that consecutive threads write the
// consecutive positions of one digit's run.
__global__ void __launch_bounds__(kSortThreads) k_sort_scatter(const uint32_t* __restrict__ keys,
                                                                const uint32_t* __restrict__ vals, uint32_t n,
                                                                int shift, int dbits,
                                                                const uint32_t* __restrict__ offs,
                                                                uint32_t* __restrict__ okeys,
                                                                uint32_t* __restrict__ ovals,
                                                                uint32_t* __restrict__ status) {
    pdl_wait();
    __shared__ uint16_t wh[kSortThreads / 32][kMaxBuckets];  // per-warp counts, then offsets
    __shared__ uint32_t boff[kMaxBuckets];                   // global start of this tile's digit d
    __shared__ uint32_t lstart[kMaxBuckets];                 // tile-local start of digit d
    __shared__ uint32_t sk[kSortTile], sv[kSortTile];
    const uint32_t nbk = 1u << dbits, mask = nbk - 1u;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t d = threadIdx.x; d < nbk; d += kSortThreads) {
        for (int w = 0; w < kSortThreads / 32; ++w) wh[w][d] = 0;
        boff[d] = offs[d * gridDim.x + blockIdx.x];
    }
    __syncthreads();
    const uint32_t tile0 = blockIdx.x * kSortTile;
    uint32_t base = tile0 + warp * (kItems * 32);
    uint32_t k[kItems], v[kItems], rk[kItems];
    uint32_t lt = (1u << lane) - 1u;
    for (int r = 0; r < kItems; ++r) {
        uint32_t i = base + r * 32 + lane;
        bool ok = i < n;
        k[r] = ok ? keys[i] : 0u;
        v[r] = ok ? vals[i] : 0u;
        uint32_t d = ok ? (k[r] >> shift) & mask : kMaxBuckets;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t before = ok ? wh[warp][d] : 0u;
        __syncwarp();
        if (ok && (peers & lt) == 0) wh[warp][d] = uint16_t(before + uint32_t(__popc(peers)));
        __syncwarp();
        rk[r] = before + uint32_t(__popc(peers & lt));
    }
    __syncthreads();
    // per digit: warp offsets inside the digit, and the digit's tile count;
    // then the tile-local start of each digit (digits split evenly over threads)
    const uint32_t per = (nbk + kSortThreads - 1) / kSortThreads;
    const uint32_t d0 = min(threadIdx.x * per, nbk), d1 = min(d0 + per, nbk);
    uint32_t mine = 0;
    for (uint32_t d = d0; d < d1; ++d) {
        uint32_t run = 0;
        for (int w = 0; w < kSortThreads / 32; ++w) {
            uint32_t c = wh[w][d];
            wh[w][d] = uint16_t(run);
            run += c;
        }
        lstart[d] = run;
        mine += run;
    }
    uint32_t tot;
    uint32_t ex = block_exclusive_scan(mine, &tot);
    for (uint32_t d = d0; d < d1; ++d) {
        uint32_t c = lstart[d];
        lstart[d] = ex;
        ex += c;
    }
    __syncthreads();
    for (int r = 0; r < kItems; ++r) {
        uint32_t i = base + r * 32 + lane;
        if (i >= n) continue;
        uint32_t d = (k[r] >> shift) & mask;
        uint32_t lp = lstart[d] + wh[warp][d] + rk[r];
        sk[lp] = k[r];
        sv[lp] = v[r];
    }
    __syncthreads();
    const uint32_t cnt = n - tile0 < uint32_t(kSortTile) ? n - tile0 : uint32_t(kSortTile);
    for (uint32_t q = threadIdx.x; q < cnt; q += kSortThreads) {
        uint32_t key = sk[q];
        uint32_t d = (key >> shift) & mask;
        uint32_t pos = boff[d] + (q - lstart[d]);
        if (!APIC_IN_BOUNDS(pos, n, status)) continue;
        okeys[pos] = key;
        ovals[pos] = sv[q];
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
    // Morton order is monotone in x and y, so the largest key is that of the
    // far corner (sides are limited to 65536, so 16 bits per axis suffice).
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

// Digit width of an LSD sort over `bits` key bits: the fewest passes of at
// most kMaxDigitBits bits, split as evenly as possible.
static int digit_bits(int bits) {
    if (bits <= 0) return 0;
    int passes = (bits + kMaxDigitBits - 1) / kMaxDigitBits;
    return (bits + passes - 1) / passes;
}

static cudaError_t lsd_passes(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt,
                              uint32_t* hist, uint32_t* scan_tmp, uint32_t n, int bits, int dbits, cudaStream_t st,
                              bool pdl, uint32_t** keys_out, uint32_t** vals_out, uint32_t* status) {
    uint32_t nb = div_up(n, kSortTile);
    uint32_t* k_in = keys;
    uint32_t* v_in = vals;
    uint32_t* k_out = keys_alt;
    uint32_t* v_out = vals_alt;
    for (int shift = 0; dbits > 0 && shift < bits; shift += dbits) {
        launch(pdl, k_sort_hist, nb, kSortThreads, 0, st, static_cast<const uint32_t*>(k_in), n, shift, dbits, hist);
        cudaError_t e = exclusive_scan_u32(hist, (1u << dbits) * nb, scan_tmp, st);
        if (e != cudaSuccess) return e;
        launch(pdl, k_sort_scatter, nb, kSortThreads, 0, st, static_cast<const uint32_t*>(k_in),
               static_cast<const uint32_t*>(v_in), n, shift, dbits, static_cast<const uint32_t*>(hist), k_out, v_out,
               status);
        std::swap(k_in, k_out);
        std::swap(v_in, v_out);
    }
    *keys_out = k_in;
    *vals_out = v_in;
    return cudaGetLastError();
}

uint32_t sort_hist_words(uint32_t n) { return kMaxBuckets * div_up(n > 0 ? n : 1, kSortTile); }
uint32_t sort_scan_words(uint32_t n) { return div_up(sort_hist_words(n), 1024) + 1; }

cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, uint32_t* hist,
                             uint32_t* scan_tmp, uint32_t n, int bits, cudaStream_t st, bool pdl,
                             uint32_t** keys_out, uint32_t** vals_out, uint32_t* status) {
    *keys_out = keys;
    *vals_out = vals;
    if (n == 0) return cudaSuccess;
    return lsd_passes(keys, vals, keys_alt, vals_alt, hist, scan_tmp, n, bits, digit_bits(bits), st, pdl, keys_out,
                      vals_out, status);
}

bool radix_sort_in_alt(int bits) {
    int d = digit_bits(bits);
    int passes = d > 0 ? (bits + d - 1) / d : 0;
    return passes % 2 == 1;
}

cudaError_t launch_sort(Scene& s) {
    if (s.n == 0) return cudaSuccess;
    float max_x = float(s.W > 0 ? s.W - 1 : 0), max_y = float(s.H > 0 ? s.H - 1 : 0);
    launch(s.use_pdl, k_morton_keys, div_up(s.n, 1024), 256, 0, s.stream, s.pp, s.n, s.dx, max_x, max_y, s.keys,
           s.vals);
    // the sorted pairs stay where the last pass wrote them (no copy back)
    uint32_t *k_res, *v_res;
    cudaError_t e = radix_sort_pairs(s.keys, s.vals, s.keys_alt, s.vals_alt, s.sort_hist, s.sort_scan_tmp, s.n,
                                     key_bits(s), s.stream, s.use_pdl, &k_res, &v_res, &s.ctl->status);
    if (e != cudaSuccess) return e;
    return launch_permute(s, v_res);
}

// Where launch_sort leaves the sorted pairs of a scene (the number of digit
// passes is fixed by the grid size).
bool sort_result_in_alt(const Scene& s) { return radix_sort_in_alt(key_bits(s)); }

// Stable LSD sort of (keys, vals)[0..n) over the low `bits` key bits in 8-bit
// digits, with all intermediate storage supplied by the caller:
// keys_alt/vals_alt (n words each), hist (256 * ceil(n / 2048) words) and
// scan_tmp (ceil(hist / 1024) words).  The sorted pairs end in keys/vals.
cudaError_t radix_sort_pairs_in(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, uint32_t* hist,
                                uint32_t* scan_tmp, uint32_t n, int bits, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    uint32_t *k_res, *v_res;
    cudaError_t e = lsd_passes(keys, vals, keys_alt, vals_alt, hist, scan_tmp, n, bits, bits > 0 ? 8 : 0, st,
                               st != nullptr, &k_res, &v_res, nullptr);
    if (e != cudaSuccess) return e;
    if (k_res != keys) {
        cudaMemcpyAsync(keys, k_res, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(vals, v_res, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st);
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
