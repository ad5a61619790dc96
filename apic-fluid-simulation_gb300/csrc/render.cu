// render.cu — headless particle splatting into a device RGBA8 frame.
//
// Restates the particle view of the reference GUI without a graphics API:
// render_particles (src/main.rs:207-277) and make_circle_texture (:73-101).
// Every particle with finite coordinates inside the frame plus a margin is
// drawn, in particle order, as a 2R x 2R pixel quad textured with a 32 x 32
// anti-aliased disc (alpha 255 inside radius 15, a linear ramp to 0 at 16),
// tinted by speed (r = min(0.01 |v|^2, 1), g = 0.5, b = 1 - r/2) and alpha
// blended over the frame (src_alpha, 1 - src_alpha) the way a draw call blends
// into an RGBA8 framebuffer: each blend is rounded back to 8 bits before the
// next particle's.  RenderStats (valid / NaN / out-of-bounds counts, :39-43,
// :226-245), the pick of the nearest particle to a point (:247-256) and the
// fluid volume of the HUD (:461-468) come with the frame.
//
// The GL pipeline's fixed-function steps are stated here as plain arithmetic:
// a pixel is covered when its centre lies in [x0, x0 + 2R) x [y0, y0 + 2R)
// (the top-left fill rule), the texture is sampled bilinearly with texel
// centres at (i + 0.5) / 32 and clamp-to-edge addressing (macroquad's default
// linear filter and clamp wrap; the texel coordinate is
// (pixel centre - quad corner) * (32 / 2R) - 0.5), and the blend runs in float
// on 8-bit framebuffer values.  Texture hardware quantises its filter weights, so a
// real GL frame may differ from this one by a unit in the last bit; the CPU
// oracle states the same arithmetic and the GPU frame matches it exactly.
//
// GPU form (ordered splatting, the tile-binning scheme of sort-based
// rasterisers): the frame is cut into 16 x 16 pixel tiles; each particle emits
// one (tile, particle) pair per tile its quad touches (at most 2 x 2 for a
// quad of at most 16 pixels), a stable radix sort by tile keeps particle order
// inside each tile, and one CTA per tile blends its list in that order with
// one thread per pixel, so every pixel sees the sequence of blends the
// reference's draw loop produces.
#include <cuda_runtime.h>

#include <cmath>

#include "apic_device.cuh"
#include "apic_internal.h"

namespace apic {

namespace {

constexpr uint32_t kTile = 16;                  // tile side in pixels (one CTA, one thread per pixel)
constexpr uint32_t kTileThreads = kTile * kTile;
constexpr int kTex = 32;                        // circle texture side (make_circle_texture)

struct RenderCounters {
    uint32_t valid, nan, oob, pad;
    unsigned long long pick;  // (bits of squared distance << 32) | particle; ~0: none
};

__device__ __forceinline__ uint32_t warp_count(bool p) { return __popc(__ballot_sync(0xffffffffu, p)); }

// Alpha of texel (x, y) of the 32 x 32 disc (src/main.rs:77-93).
__device__ __forceinline__ uint32_t circle_alpha(int x, int y) {
    const float radius = float(kTex) / 2.0f;
    const float dx = float(x) - radius + 0.5f;
    const float dy = float(y) - radius + 0.5f;
    const float dist = sqrtf(dx * dx + dy * dy);
    if (dist < radius - 1.0f) return 255u;
    if (dist < radius) {
        const float a = (radius - dist) * 255.0f;  // `as u8`: truncation, saturating at 0..255
        return a >= 255.0f ? 255u : (a > 0.0f ? uint32_t(a) : 0u);
    }
    return 0u;
}

// Per particle: counters, pick candidate, quad corner + tint, and the (tile,
// particle) pairs of its quad; slots of tiles it does not touch get the key
// `ntiles`, which sorts after every real tile.
__global__ void __launch_bounds__(256) k_splat_bin(const PartPtrs* __restrict__ pp, uint32_t n, RenderParamsDev p,
                                                   float4* __restrict__ quad, uint32_t* __restrict__ keys,
                                                   uint32_t* __restrict__ vals, RenderCounters* __restrict__ cnt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < n;
    float x = 0.0f, y = 0.0f, vx = 0.0f, vy = 0.0f;
    if (live) {
        x = pp->f[PX][i];
        y = pp->f[PY][i];
        vx = pp->f[VX][i];
        vy = pp->f[VY][i];
    }
    const bool finite = live && isfinite(x) && isfinite(y);
    const float draw_x = x * p.scale;
    const float draw_y = p.fh - y * p.scale;
    const bool oob = finite && (draw_x < -p.margin || draw_x > p.fw + p.margin || draw_y < -p.margin ||
                                draw_y > p.fh + p.margin);
    const bool valid = finite && !oob;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nv = warp_count(valid), nn = warp_count(live && !finite), no = warp_count(oob);
    if (lane == 0) {
        if (nv) atomicAdd(&cnt->valid, nv);
        if (nn) atomicAdd(&cnt->nan, nn);
        if (no) atomicAdd(&cnt->oob, no);
    }
    if (!live) return;
    uint32_t k0 = p.ntiles, k1 = p.ntiles, k2 = p.ntiles, k3 = p.ntiles;
    if (valid) {
        if (p.pick_r2 >= 0.0f) {
            const float dx = draw_x - p.pick_x;
            const float dy = draw_y - p.pick_y;
            const float d2 = dx * dx + dy * dy;
            if (d2 <= p.pick_r2)
                atomicMin(&cnt->pick, (static_cast<unsigned long long>(__float_as_uint(d2)) << 32) | i);
        }
        const float speed_sq = vx * vx + vy * vy;
        const float r = fminf(speed_sq * 0.01f, 1.0f);
        const float qx = draw_x - p.radius, qy = draw_y - p.radius;
        quad[i] = make_float4(qx, qy, r, 0.0f);
        // tiles of the pixels whose centres can fall in [q, q + 2R): a span
        // one pixel wider on each side (at most 2R + 2 <= 16 pixels, so at
        // most two tiles per axis); the raster test per pixel is exact
        const int tx0 = max(int(floorf((qx - 1.0f) / float(kTile))), 0);
        const int tx1 = min(int(floorf((qx + p.size + 1.0f) / float(kTile))), int(p.ntx) - 1);
        const int ty0 = max(int(floorf((qy - 1.0f) / float(kTile))), 0);
        const int ty1 = min(int(floorf((qy + p.size + 1.0f) / float(kTile))), int(p.nty) - 1);
        if (tx0 <= tx1 && ty0 <= ty1) {  // else the quad lies outside the frame
            const uint32_t t = uint32_t(ty0) * p.ntx + uint32_t(tx0);
            const bool two_x = tx1 > tx0, two_y = ty1 > ty0;
            k0 = t;
            if (two_x) k1 = t + 1;
            if (two_y) k2 = t + p.ntx;
            if (two_x && two_y) k3 = t + p.ntx + 1;
        }
    }
    *reinterpret_cast<uint4*>(keys + size_t(i) * 4) = make_uint4(k0, k1, k2, k3);
    *reinterpret_cast<uint4*>(vals + size_t(i) * 4) = make_uint4(i, i, i, i);
}

// First and one-past-last sorted pair of every tile (both zeroed before).
__global__ void k_tile_ranges(const uint32_t* __restrict__ keys, uint32_t m, uint32_t ntiles,
                              uint32_t* __restrict__ start, uint32_t* __restrict__ end) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const uint32_t k = keys[j];
    if (k >= ntiles) return;
    if (j == 0 || keys[j - 1] != k) start[k] = j;
    if (j + 1 == m || keys[j + 1] != k) end[k] = j + 1;
}

// d8: the 256 values k / 255 (an 8-bit channel as a float).
__device__ __forceinline__ uint32_t blend8(float c, float a, uint32_t dst, const float* d8) {
    const float d = d8[dst];
    const float o = c * a + d * (1.0f - a);
    const float q = o * 255.0f + 0.5f;
    return q >= 255.0f ? 255u : (q > 0.0f ? uint32_t(q) : 0u);
}

// One CTA per 16 x 16 tile, one thread per pixel: blend the tile's quads in
// particle order.
__global__ void __launch_bounds__(kTileThreads) k_splat_raster(const uint32_t* __restrict__ vals,
                                                              const uint32_t* __restrict__ start,
                                                              const uint32_t* __restrict__ end,
                                                              const float4* __restrict__ quad, RenderParamsDev p,
                                                              uint32_t* __restrict__ frame) {
    __shared__ float tex[kTex * kTex];
    __shared__ float d8[256];
    __shared__ float4 ent[kTileThreads];
    for (int t = threadIdx.x; t < kTex * kTex; t += kTileThreads)
        tex[t] = float(circle_alpha(t % kTex, t / kTex)) / 255.0f;
    d8[threadIdx.x] = float(threadIdx.x) / 255.0f;
    const uint32_t tile = blockIdx.x;
    const uint32_t px = (tile % p.ntx) * kTile + (threadIdx.x % kTile);
    const uint32_t py = (tile / p.ntx) * kTile + (threadIdx.x / kTile);
    const float cx = float(px) + 0.5f, cy = float(py) + 0.5f;
    uint32_t dr = p.bg & 0xFFu, dg = (p.bg >> 8) & 0xFFu, db = (p.bg >> 16) & 0xFFu;
    const uint32_t b0 = start[tile], b1 = end[tile];
    __syncthreads();
    for (uint32_t base = b0; base < b1; base += kTileThreads) {
        const uint32_t j = base + threadIdx.x;
        if (j < b1) ent[threadIdx.x] = quad[vals[j]];
        __syncthreads();
        const uint32_t cnt = min(kTileThreads, b1 - base);
        for (uint32_t e = 0; e < cnt; ++e) {
            const float4 q = ent[e];
            if (!(q.x <= cx && cx < q.x + p.size && q.y <= cy && cy < q.y + p.size)) continue;
            const float u = (cx - q.x) * p.tex_scale - 0.5f;
            const float v = (cy - q.y) * p.tex_scale - 0.5f;
            const float fu = floorf(u), fv = floorf(v);
            const float wu = u - fu, wv = v - fv;
            const int iu = int(fu), iv = int(fv);
            const int u0 = min(max(iu, 0), kTex - 1), u1 = min(max(iu + 1, 0), kTex - 1);
            const int v0 = min(max(iv, 0), kTex - 1), v1 = min(max(iv + 1, 0), kTex - 1);
            const float top = tex[v0 * kTex + u0] * (1.0f - wu) + tex[v0 * kTex + u1] * wu;
            const float bot = tex[v1 * kTex + u0] * (1.0f - wu) + tex[v1 * kTex + u1] * wu;
            const float a = top * (1.0f - wv) + bot * wv;
            const float r = q.z;
            dr = blend8(r, a, dr, d8);
            dg = blend8(0.5f, a, dg, d8);
            db = blend8(1.0f - r * 0.5f, a, db, d8);
        }
        __syncthreads();
    }
    if (px < p.width && py < p.height) frame[size_t(py) * p.width + px] = dr | (dg << 8) | (db << 16) | (0xFFu << 24);
}

template <typename T>
cudaError_t grow(T** ptr, size_t* cap, size_t count) {
    if (*cap >= count) return cudaSuccess;
    if (*ptr) cudaFree(*ptr);
    *ptr = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(ptr), count * sizeof(T));
    if (e == cudaSuccess) *cap = count;
    return e;
}

int bit_length(uint32_t v) {
    int b = 0;
    while (b < 32 && (v >> b)) ++b;
    return b;
}

}  // namespace

// Device buffers of the splatting pass, grown on demand.
struct RenderBuffers {
    uint32_t* frame = nullptr;
    size_t frame_cap = 0;
    uint32_t width = 0, height = 0;  // of the last frame
    float4* quad = nullptr;
    size_t quad_cap = 0;
    uint32_t *keys = nullptr, *vals = nullptr, *keys_alt = nullptr, *vals_alt = nullptr;
    size_t keys_cap = 0, vals_cap = 0, keys_alt_cap = 0, vals_alt_cap = 0;
    uint32_t *hist = nullptr, *scan_tmp = nullptr;
    size_t hist_cap = 0, scan_cap = 0;
    uint32_t *start = nullptr, *end = nullptr;
    size_t start_cap = 0, end_cap = 0;
    RenderCounters* cnt = nullptr;
    RenderCounters* cnt_host = nullptr;
};

void free_render(Scene& s) {
    RenderBuffers* b = s.render;
    if (!b) return;
    void* ptrs[] = {b->frame, b->quad, b->keys, b->vals, b->keys_alt, b->vals_alt, b->hist, b->scan_tmp,
                    b->start, b->end, b->cnt};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    if (b->cnt_host) cudaFreeHost(b->cnt_host);
    delete b;
    s.render = nullptr;
}

cudaError_t render_frame(Scene& s, const RenderParamsDev& p, RenderResult* out) {
    if (!s.render) s.render = new RenderBuffers();
    RenderBuffers& b = *s.render;
    const size_t pixels = size_t(p.width) * p.height;
    const size_t m = size_t(s.n) * 4;
    const uint32_t sort_blocks = div_up(m, kSortTile);
    const size_t hist_words = size_t(256) * (sort_blocks ? sort_blocks : 1);
    cudaError_t e;
    if ((e = grow(&b.frame, &b.frame_cap, pixels)) != cudaSuccess) return e;
    if ((e = grow(&b.quad, &b.quad_cap, size_t(s.n ? s.n : 1))) != cudaSuccess) return e;
    if ((e = grow(&b.keys, &b.keys_cap, m ? m : 1)) != cudaSuccess) return e;
    if ((e = grow(&b.vals, &b.vals_cap, m ? m : 1)) != cudaSuccess) return e;
    if ((e = grow(&b.keys_alt, &b.keys_alt_cap, m ? m : 1)) != cudaSuccess) return e;
    if ((e = grow(&b.vals_alt, &b.vals_alt_cap, m ? m : 1)) != cudaSuccess) return e;
    if ((e = grow(&b.hist, &b.hist_cap, hist_words)) != cudaSuccess) return e;
    if ((e = grow(&b.scan_tmp, &b.scan_cap, size_t(div_up(hist_words, 1024)) + 1)) != cudaSuccess) return e;
    if ((e = grow(&b.start, &b.start_cap, size_t(p.ntiles))) != cudaSuccess) return e;
    if ((e = grow(&b.end, &b.end_cap, size_t(p.ntiles))) != cudaSuccess) return e;
    if (!b.cnt && (e = cudaMalloc(&b.cnt, sizeof(RenderCounters))) != cudaSuccess) return e;
    if (!b.cnt_host && (e = cudaMallocHost(&b.cnt_host, sizeof(RenderCounters))) != cudaSuccess) return e;
    b.width = p.width;
    b.height = p.height;

    cudaStream_t st = s.stream;
    RenderCounters init{0u, 0u, 0u, 0u, ~0ull};
    *b.cnt_host = init;
    if ((e = cudaMemcpyAsync(b.cnt, b.cnt_host, sizeof(RenderCounters), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return e;
    cudaMemsetAsync(b.start, 0, sizeof(uint32_t) * p.ntiles, st);
    cudaMemsetAsync(b.end, 0, sizeof(uint32_t) * p.ntiles, st);
    if (s.n) {
        k_splat_bin<<<div_up(s.n, 256), 256, 0, st>>>(s.pp, s.n, p, b.quad, b.keys, b.vals, b.cnt);
        if ((e = radix_sort_pairs_in(b.keys, b.vals, b.keys_alt, b.vals_alt, b.hist, b.scan_tmp, uint32_t(m),
                                     bit_length(p.ntiles), st)) != cudaSuccess)
            return e;
        k_tile_ranges<<<div_up(m, 256), 256, 0, st>>>(b.keys, uint32_t(m), p.ntiles, b.start, b.end);
    }
    k_splat_raster<<<p.ntiles, kTileThreads, 0, st>>>(b.vals, b.start, b.end, b.quad, p, b.frame);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(b.cnt_host, b.cnt, sizeof(RenderCounters), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    out->valid = b.cnt_host->valid;
    out->nan = b.cnt_host->nan;
    out->oob = b.cnt_host->oob;
    out->picked = b.cnt_host->pick == ~0ull ? -1 : int64_t(b.cnt_host->pick & 0xFFFFFFFFull);
    // bin + ranges + raster, and per 8-bit sort pass: histogram, three scan
    // kernels, scatter
    out->kernels = s.n ? 3u + 5u * uint32_t((bit_length(p.ntiles) + 7) / 8) : 1u;
    return cudaSuccess;
}

const uint32_t* render_frame_ptr(const Scene& s, uint32_t* width, uint32_t* height) {
    if (!s.render || !s.render->frame || s.render->width == 0) return nullptr;
    *width = s.render->width;
    *height = s.render->height;
    return s.render->frame;
}

}  // namespace apic
