// grid.cu — MAC-grid and cell stages of the substep.
//
//   k_faces          normalise the P2G sums (src/apic.rs:1428-1459), add the
//                    external force (:1607-1612) and gravity on faces next to
//                    fluid (:1614-1625); one thread per face, fused.
//   k_compact_*      fluid mask clean-up (:1463-1464) and the ascending list of
//                    non-zero mask words of a level (the GPU form of the
//                    reference's fluid/red/black index lists, :1461-1494 and
//                    :1526-1553), with the fluid-cell count and the last fluid
//                    cell that the padded list duplicates (:1487-1494).
//   k_smooth_density three Jacobi passes over fluid cells (:1653-1685).
//   k_laplacian      divergence, ghost-fluid diagonal, +x/+y couplings and
//                    the density-correction right-hand side (:1698-1784).
//   k_coarsen        one multigrid level from its finer level (:1499-1602).
//   k_gradient       pressure projection per face (:1958-2055), fused with the
//                    post-force add (:2453-2458).
//   k_extrapolate2   two Jacobi sweeps of velocity extrapolation for u and v
//                    in shared-memory tiles (:2266-2350).
//
// Cell stages run one warp per non-zero 32-bit mask word ("segment"): lane k
// owns raw cell 32*word + k, so every field access of a warp is one 128-byte
// line.  Neighbour reads are gated by the neighbour's fluid bit, which equals
// the reference's reads of zero-filled or zero-coefficient entries.
#include <cuda_runtime.h>

#include "apic_device.cuh"
#include "apic_internal.h"

namespace apic {
namespace {

constexpr int kCompactWords = 1024;  // mask words per compaction block

__global__ void __launch_bounds__(256) k_faces(uint32_t uf, uint32_t vf, int W, int H, const float* __restrict__ acc_u,
                                               const float* __restrict__ acc_uw, const float* __restrict__ acc_v,
                                               const float* __restrict__ acc_vw, float* __restrict__ u,
                                               float* __restrict__ v, uint8_t* __restrict__ valid_u,
                                               uint8_t* __restrict__ valid_v, const float* __restrict__ ext_u,
                                               const float* __restrict__ ext_v, const uint32_t* __restrict__ fluid,
                                               const uint32_t* __restrict__ obstacle, const Ctl* __restrict__ ctl,
                                               float gravity, int normalize, int forces, int apply_gravity) {
    pdl_wait();
    uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= uf + vf) return;
    const float dt = ctl->dt;
    const bool ext = forces && ctl->has_ext;
    if (f < uf) {
        float val;
        if (normalize) {
            float w = acc_uw[f];
            val = 0.0f;
            uint8_t ok = 0;
            if (w > 0.0f) { val = acc_u[f] / w; ok = 1; }
            valid_u[f] = ok;
        } else {
            val = u[f];
        }
        if (ext) val += ext_u[f] * dt;
        u[f] = val;
    } else {
        uint32_t g = f - uf;
        float val;
        if (normalize) {
            float w = acc_vw[g];
            val = 0.0f;
            uint8_t ok = 0;
            if (w > 0.0f) { val = acc_v[g] / w; ok = 1; }
            valid_v[g] = ok;
        } else {
            val = v[g];
        }
        if (ext) val += ext_v[g] * dt;
        if (apply_gravity) {
            int x = int(g % uint32_t(W)), y = int(g / uint32_t(W));
            // fluid bits net of obstacles, whether or not the mask has been cleaned yet
            uint32_t fb = fluid_xy(fluid, x, y - 1, W, H) & (1u - obstacle_xy(obstacle, x, y - 1, W, H));
            uint32_t ft = fluid_xy(fluid, x, y, W, H) & (1u - obstacle_xy(obstacle, x, y, W, H));
            if (fb || ft) val += gravity * dt;
        }
        v[g] = val;
    }
}

// Block b of the compaction owns mask words [b*1024, b*1024 + 1024).
__device__ __forceinline__ uint32_t load_clean_word(uint32_t* fluid, const uint32_t* obstacle, uint32_t w, uint32_t words,
                                                    bool write_back) {
    if (w >= words) return 0u;
    uint32_t m = fluid[w];
    if (obstacle) {
        uint32_t c = m & ~obstacle[w];
        if (write_back && c != m) fluid[w] = c;
        m = c;
    }
    return m;
}

__global__ void __launch_bounds__(256) k_compact_count(uint32_t* __restrict__ fluid, const uint32_t* __restrict__ obstacle,
                                                       uint32_t words, uint32_t* __restrict__ cnt) {
    pdl_wait();
    uint32_t nz = 0, cells = 0, last = 0;
    for (int k = 0; k < 4; ++k) {
        uint32_t w = blockIdx.x * kCompactWords + threadIdx.x * 4 + k;
        uint32_t m = load_clean_word(fluid, obstacle, w, words, true);
        if (m) { nz++; cells += __popc(m); last = max(last, w + 1); }
    }
    __shared__ uint32_t s[3][256];
    s[0][threadIdx.x] = nz; s[1][threadIdx.x] = cells; s[2][threadIdx.x] = last;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            s[0][threadIdx.x] += s[0][threadIdx.x + o];
            s[1][threadIdx.x] += s[1][threadIdx.x + o];
            s[2][threadIdx.x] = max(s[2][threadIdx.x], s[2][threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        cnt[3 * blockIdx.x + 0] = s[0][0];
        cnt[3 * blockIdx.x + 1] = s[1][0];
        cnt[3 * blockIdx.x + 2] = s[2][0];
    }
}

__device__ __forceinline__ uint32_t scan_1024(uint32_t v, uint32_t* total) {
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

// Segment list of one level (ascending non-zero mask words): block b writes
// its words after those of blocks [0, b), whose counts (k_compact_count) it
// sums itself; the last block also records the level's totals in Ctl (and,
// on the base level, the fluid-cell count, the last fluid cell and the
// padding of the reference's fluid list to a multiple of 8).
__global__ void __launch_bounds__(256) k_compact_write(const uint32_t* __restrict__ fluid, uint32_t words,
                                                       const uint32_t* __restrict__ cnt, uint32_t* __restrict__ seg,
                                                       uint32_t W, int level, Ctl* __restrict__ ctl) {
    pdl_wait();
    const uint32_t nb = gridDim.x, b0 = blockIdx.x;
    const bool last_block = b0 + 1 == nb;
    uint32_t before = 0, total = 0, cells = 0, lastw = 0;
    for (uint32_t b = threadIdx.x; b < (last_block ? nb : b0); b += 256) {
        const uint32_t c = cnt[3 * b];
        before += b < b0 ? c : 0u;
        total += c;
        cells += cnt[3 * b + 1];
        lastw = max(lastw, cnt[3 * b + 2]);
    }
    __shared__ uint32_t red[4][256];
    red[0][threadIdx.x] = before;
    red[1][threadIdx.x] = total;
    red[2][threadIdx.x] = cells;
    red[3][threadIdx.x] = lastw;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            red[0][threadIdx.x] += red[0][threadIdx.x + o];
            red[1][threadIdx.x] += red[1][threadIdx.x + o];
            red[2][threadIdx.x] += red[2][threadIdx.x + o];
            red[3][threadIdx.x] = max(red[3][threadIdx.x], red[3][threadIdx.x + o]);
        }
        __syncthreads();
    }
    uint32_t m[4], nz = 0;
    for (int k = 0; k < 4; ++k) {
        uint32_t w = b0 * kCompactWords + threadIdx.x * 4 + k;
        m[k] = w < words ? fluid[w] : 0u;
        nz += m[k] ? 1u : 0u;
    }
    uint32_t tot;
    uint32_t off = red[0][0] + scan_1024(nz, &tot);
    for (int k = 0; k < 4; ++k)
        if (m[k]) seg[off++] = b0 * kCompactWords + threadIdx.x * 4 + k;
    if (!last_block || threadIdx.x != 0) return;
    ctl->seg_count[level] = red[1][0];
    if (level == 0) {
        const uint32_t f = red[2][0], lw = red[3][0];
        ctl->fluid_cells = f;
        if (f > 0 && lw > 0) {
            const uint32_t mw = fluid[lw - 1];
            ctl->last_fluid = (lw - 1) * 32u + (31u - uint32_t(__clz(mw))) + W;
        } else {
            ctl->last_fluid = 0;
        }
        ctl->pad_count = (8u - f % 8u) % 8u;
    }
}

// Smoothed density as the consumers see it: the three-pass result at fluid
// cells, the P2G density elsewhere (src/apic.rs:1649-1685 smooths fluid cells only).
__device__ __forceinline__ float smoothed_at(const float* sm, const float* dens, const uint32_t* fluid, uint32_t c) {
    return bit_at(fluid, c) ? sm[c] : dens[c];
}
// Same, for a cell index that can fall one row past the grid when a caller
// opens the solid border (the reference reads past its array there).
__device__ __forceinline__ float smoothed_guarded(const float* sm, const float* dens, const uint32_t* fluid,
                                                  uint32_t c, uint32_t cells) {
    return c < cells ? smoothed_at(sm, dens, fluid, c) : 0.0f;
}

__global__ void __launch_bounds__(kSegBlock) k_smooth_density(const uint32_t* __restrict__ fluid,
                                                               const uint32_t* __restrict__ seg,
                                                               const Ctl* __restrict__ ctl, uint32_t W, uint32_t cells,
                                                               const float* __restrict__ src, float* __restrict__ dst) {
    pdl_wait();
    const uint32_t nseg = ctl->seg_count[0];
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nseg; s += nw) {
        uint32_t word = seg[s];
        uint32_t bits = fluid[word];
        if (!((bits >> lane) & 1u)) continue;
        long long raw = (long long)word * 32 + lane;
        float fl = float(fluid_raw(fluid, raw - 1, cells)), fr = float(fluid_raw(fluid, raw + 1, cells));
        float fb = float(fluid_raw(fluid, raw - (long long)W, cells)), ft = float(fluid_raw(fluid, raw + (long long)W, cells));
        float sum = src[raw] * 4.0f;
        float weight = 4.0f;
        if (fl != 0.0f) sum += src[raw - 1];
        if (fr != 0.0f) sum += src[raw + 1];
        if (fb != 0.0f) sum += src[raw - W];
        if (ft != 0.0f) sum += src[raw + W];
        weight += fl + fr + fb + ft;
        dst[raw] = sum / weight;
    }
}

__global__ void __launch_bounds__(kSegBlock) k_laplacian(const uint32_t* __restrict__ fluid,
                                                          const uint32_t* __restrict__ obstacle,
                                                          const uint32_t* __restrict__ seg, const Ctl* __restrict__ ctl,
                                                          uint32_t W, uint32_t cells, float dx,
                                                          const float* __restrict__ u, const float* __restrict__ v,
                                                          const float* __restrict__ sm, const float* __restrict__ dens,
                                                          float* __restrict__ res, float* __restrict__ diag_o,
                                                          float* __restrict__ inv_o, float* __restrict__ px_o,
                                                          float* __restrict__ py_o) {
    pdl_wait();
    const uint32_t nseg = ctl->seg_count[0];
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const float target = 9.0f;
    const float noise = target * 1.15f;
    const float corr = 0.1f;
    for (uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nseg; s += nw) {
        uint32_t word = seg[s];
        uint32_t bits = fluid[word];
        if (!((bits >> lane) & 1u)) continue;
        long long raw = (long long)word * 32 + lane;
        uint32_t fi = uint32_t(raw) + W;
        uint32_t gx = uint32_t(raw) % W, gy = uint32_t(raw) / W;
        uint32_t ui = gy * (W + 1) + gx;
        float ul = u[ui], ur = u[ui + 1], vb = v[raw], vt = v[raw + W];
        uint32_t nol = 1u - obstacle_raw(obstacle, raw - 1, cells), nor = 1u - obstacle_raw(obstacle, raw + 1, cells);
        uint32_t nob = 1u - obstacle_raw(obstacle, raw - (long long)W, cells);
        uint32_t not_ = 1u - obstacle_raw(obstacle, raw + (long long)W, cells);
        ul *= float(nol);
        ur *= float(nor);
        vb *= float(nob);
        vt *= float(not_);
        float div = (ur - ul) + (vt - vb);
        float rc = sm[raw];
        float excess = fminf(fmaxf(rc - noise, 0.0f), target);
        uint32_t fl = fluid_raw(fluid, raw - 1, cells), fr = fluid_raw(fluid, raw + 1, cells);
        uint32_t fb = fluid_raw(fluid, raw - (long long)W, cells), ft = fluid_raw(fluid, raw + (long long)W, cells);
        float diag = 0.0f, px = 0.0f, py = 0.0f;
        if (nol) {
            if (fl) diag += 1.0f;
            else diag += 1.0f / theta(smoothed_at(sm, dens, fluid, uint32_t(raw - 1)), rc, target);
        }
        if (nor) {
            if (fr) { diag += 1.0f; px = -1.0f; }
            else diag += 1.0f / theta(smoothed_at(sm, dens, fluid, uint32_t(raw + 1)), rc, target);
        }
        if (nob) {
            if (fb) diag += 1.0f;
            else diag += 1.0f / theta(smoothed_at(sm, dens, fluid, uint32_t(raw - W)), rc, target);
        }
        if (not_) {
            if (ft) { diag += 1.0f; py = -1.0f; }
            else diag += 1.0f / theta(smoothed_at(sm, dens, fluid, uint32_t(raw + W)), rc, target);
        }
        res[fi] = -div * dx + excess * corr * dx * dx;
        px_o[fi] = px;
        py_o[fi] = py;
        diag_o[fi] = diag;
        inv_o[fi] = diag > 1e-6f ? 1.0f / diag : 0.0f;
    }
}

// One coarse mask word of level c from its finer level f (src/apic.rs:
// 1499-1602), by one warp: lane = the word's cell; the word itself (an OR of
// each cell's 2 x 2 children) and, for the fluid cells, the coarse
// coefficients.
__device__ __forceinline__ void coarsen_word(const Level& f, const Level& c, uint32_t word, uint32_t lane) {
    const uint32_t raw = word * 32u + lane;
    bool on = false;
    uint32_t cx = 0, cy = 0;
    if (raw < c.cells) {
        raw_xy(raw, c.w, c.wshift, cx, cy);
        for (uint32_t dy = 0; dy < 2; ++dy)
            for (uint32_t dx = 0; dx < 2; ++dx) {
                uint32_t fx = cx * 2 + dx, fy = cy * 2 + dy;
                if (fx < f.w && fy < f.h && bit_at(f.fluid, fy * f.w + fx)) on = true;
            }
    }
    const uint32_t ballot = __ballot_sync(0xffffffffu, on);
    if (lane == 0) c.fluid[word] = ballot;
    if (!on) return;
    float diag = 0.0f, px = 0.0f, py = 0.0f;
    for (uint32_t dy = 0; dy < 2; ++dy)
        for (uint32_t dx = 0; dx < 2; ++dx) {
            uint32_t fx = cx * 2 + dx, fy = cy * 2 + dy;
            if (fx >= f.w || fy >= f.h) continue;
            uint32_t fr = fy * f.w + fx, fp = fr + f.w;
            if (bit_at(f.fluid, fr)) {
                diag += f.diag[fp];
                if (dx == 0) diag += 2.0f * f.px[fp];
                if (dy == 0) diag += 2.0f * f.py[fp];
                if (dx == 1) px += f.px[fp];
                if (dy == 1) py += f.py[fp];
            }
        }
    uint32_t cp = raw + c.w;
    float fd = diag * 0.5f;
    c.diag[cp] = fd;
    c.inv_diag[cp] = fd > 1e-6f ? 1.0f / fd : 0.0f;
    c.px[cp] = px * 0.5f;
    c.py[cp] = py * 0.5f;
}

// One coarse level from its finer level: one warp per coarse mask word.
__global__ void __launch_bounds__(256) k_coarsen(Level f, Level c) {
    pdl_wait();
    const uint32_t word = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (word >= c.words) return;  // whole warps exit together
    coarsen_word(f, c, word, threadIdx.x & 31u);
}

// Segment list of one coarse level by one CTA of kOneThreads threads (levels
// of at most kOneWords mask words): thread t takes the consecutive words
// [t k, t k + k), so a block scan of the per-thread counts gives every
// non-zero word its place in ascending order.
constexpr uint32_t kOneThreads = 1024;
constexpr uint32_t kOneWords = 8192;
__device__ __forceinline__ void compact_one(const uint32_t* __restrict__ fluid, uint32_t words, uint32_t* __restrict__ seg,
                                            int level, Ctl* __restrict__ ctl) {
    const uint32_t per = (words + kOneThreads - 1) / kOneThreads;
    const uint32_t w0 = threadIdx.x * per;
    uint32_t nz = 0;
    for (uint32_t k = 0; k < per; ++k)
        if (w0 + k < words && fluid[w0 + k]) ++nz;
    uint32_t tot;
    uint32_t off = scan_1024(nz, &tot);
    for (uint32_t k = 0; k < per; ++k)
        if (w0 + k < words && fluid[w0 + k]) seg[off++] = w0 + k;
    if (threadIdx.x == 0) ctl->seg_count[level] = tot;
}

__global__ void __launch_bounds__(kOneThreads) k_compact_one(const uint32_t* __restrict__ fluid, uint32_t words,
                                                              uint32_t* __restrict__ seg, int level, Ctl* __restrict__ ctl) {
    pdl_wait();
    compact_one(fluid, words, seg, level, ctl);
}

// The smallest levels, [first, n), by one CTA: each level's coarsening (a
// warp per mask word), then its segment list, with CTA barriers between.
struct TailLevels {
    int first, n;
    Level lv[kMaxLevels];
};
__global__ void __launch_bounds__(kOneThreads) k_coarsen_tail(TailLevels t, Ctl* __restrict__ ctl) {
    pdl_wait();
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    for (int l = t.first; l < t.n; ++l) {
        const Level& f = t.lv[l - 1];
        const Level& c = t.lv[l];
        for (uint32_t w = warp; w < c.words; w += kOneThreads / 32u) coarsen_word(f, c, w, lane);
        __syncthreads();
        compact_one(c.fluid, c.words, c.seg, l, ctl);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_gradient(uint32_t uf, uint32_t vf, int W, int H, float inv_dx,
                                                  float* __restrict__ u, float* __restrict__ v,
                                                  uint8_t* __restrict__ valid_u, uint8_t* __restrict__ valid_v,
                                                  const uint32_t* __restrict__ fluid,
                                                  const uint32_t* __restrict__ obstacle,
                                                  const float* __restrict__ p, const float* __restrict__ sm,
                                                  const float* __restrict__ dens, const float* __restrict__ post_u,
                                                  const float* __restrict__ post_v, const Ctl* __restrict__ ctl,
                                                  const double* __restrict__ p64, int do_gradient, int do_post) {
    pdl_wait();
    uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= uf + vf) return;
    const float target = 9.0f;
    const uint32_t cells = uint32_t(W) * uint32_t(H);
    const bool post = do_post && ctl->has_post;
    if (f < uf) {
        int x = int(f % uint32_t(W + 1)), y = int(f / uint32_t(W + 1));
        float val = u[f];
        if (do_gradient) {
            uint32_t lo = obstacle_xy(obstacle, x - 1, y, W, H), ro = obstacle_xy(obstacle, x, y, W, H);
            if (lo != ro) {
                val = 0.0f;
                valid_u[f] = 1;
            } else {
                uint32_t lf = fluid_xy(fluid, x - 1, y, W, H), rf = fluid_xy(fluid, x, y, W, H);
                float dp = 0.0f;
                uint32_t li = uint32_t(y * W + x - 1), ri = uint32_t(y * W + x);
                if (p64) {
                    // mixed precision: differences of the FP64 refined pressure
                    double d = 0.0;
                    if (lf && rf) d = p64[ri + W] - p64[li + W];
                    else if (lf) d = -p64[li + W] / double(theta(smoothed_guarded(sm, dens, fluid, ri, cells), sm[li], target));
                    else if (rf) d = p64[ri + W] / double(theta(smoothed_guarded(sm, dens, fluid, li, cells), sm[ri], target));
                    val -= float(d * double(inv_dx));
                } else {
                    if (lf && rf) dp = p[ri] - p[li];
                    else if (lf) dp = -p[li] / theta(smoothed_guarded(sm, dens, fluid, ri, cells), sm[li], target);
                    else if (rf) dp = p[ri] / theta(smoothed_guarded(sm, dens, fluid, li, cells), sm[ri], target);
                    val -= dp * inv_dx;
                }
            }
        }
        if (post) val += post_u[f] * ctl->dt;
        u[f] = val;
    } else {
        uint32_t g = f - uf;
        int x = int(g % uint32_t(W)), y = int(g / uint32_t(W));
        float val = v[g];
        if (do_gradient) {
            uint32_t bo = obstacle_xy(obstacle, x, y - 1, W, H), to = obstacle_xy(obstacle, x, y, W, H);
            if (bo != to) {
                val = 0.0f;
                valid_v[g] = 1;
            } else {
                uint32_t bf = fluid_xy(fluid, x, y - 1, W, H), tf = fluid_xy(fluid, x, y, W, H);
                float dp = 0.0f;
                uint32_t bi = uint32_t((y - 1) * W + x), ti = uint32_t(y * W + x);
                if (p64) {
                    double d = 0.0;
                    if (bf && tf) d = p64[ti + W] - p64[bi + W];
                    else if (bf) d = -p64[bi + W] / double(theta(smoothed_guarded(sm, dens, fluid, ti, cells), sm[bi], target));
                    else if (tf) d = p64[ti + W] / double(theta(smoothed_guarded(sm, dens, fluid, bi, cells), sm[ti], target));
                    val -= float(d * double(inv_dx));
                } else {
                    if (bf && tf) dp = p[ti] - p[bi];
                    else if (bf) dp = -p[bi] / theta(smoothed_guarded(sm, dens, fluid, ti, cells), sm[bi], target);
                    else if (tf) dp = p[ti] / theta(smoothed_guarded(sm, dens, fluid, bi, cells), sm[ti], target);
                    val -= dp * inv_dx;
                }
            }
        }
        if (post) val += post_v[g] * ctl->dt;
        v[g] = val;
    }
}

// Velocity extrapolation, two Jacobi sweeps per launch (src/apic.rs:2266-2350
// runs four, swapping buffers after each).  A CTA owns a kExTX x kExTY tile
// of one face field (u: (W+1) x H, v: W x (H+1)) and stages the tile plus a
// two-face halo in shared memory; sweep 1 runs on the halo-shrunk region,
// sweep 2 on the tile, which is written out.  A neighbour outside the field
// reads as invalid, which is exactly the reference's x > 0 / x < width /
// y > 0 / y < height guards, and every face adds its valid neighbours in the
// reference's order (x-1, x+1, y-1, y+1) before the one division, so each
// sweep's values and flags are bit-identical to a sweep over the whole grid.
constexpr int kExTX = 128, kExTY = 24, kExHalo = 2;
constexpr int kExRX = kExTX + 2 * kExHalo, kExRY = kExTY + 2 * kExHalo;

struct ExField {
    const float* in;
    const uint8_t* in_ok;
    float* out;
    uint8_t* out_ok;
    int w, h;          // faces per row, rows
    int tiles_x;       // tiles per row of tiles
};

__device__ __forceinline__ void ex_face(const float* val, const uint8_t* ok, int i, float* nv, uint8_t* nok) {
    if (ok[i]) { *nv = val[i]; *nok = 1; return; }
    float sum = 0.0f;
    uint32_t cnt = 0;
    if (ok[i - 1]) { sum += val[i - 1]; cnt++; }
    if (ok[i + 1]) { sum += val[i + 1]; cnt++; }
    if (ok[i - kExRX]) { sum += val[i - kExRX]; cnt++; }
    if (ok[i + kExRX]) { sum += val[i + kExRX]; cnt++; }
    if (cnt > 0) { *nv = sum / float(cnt); *nok = 1; }
    else { *nv = val[i]; *nok = 0; }
}

__global__ void __launch_bounds__(256) k_extrapolate2(ExField fu, ExField fv, int tiles_u) {
    __shared__ float s_val[2][kExRX * kExRY];
    __shared__ uint8_t s_ok[2][kExRX * kExRY];
    const bool is_u = int(blockIdx.x) < tiles_u;
    const ExField& F = is_u ? fu : fv;
    const int t = is_u ? int(blockIdx.x) : int(blockIdx.x) - tiles_u;
    const int x0 = (t % F.tiles_x) * kExTX - kExHalo, y0 = (t / F.tiles_x) * kExTY - kExHalo;
    pdl_wait();
    for (int i = threadIdx.x; i < kExRX * kExRY; i += blockDim.x) {
        const int gx = x0 + i % kExRX, gy = y0 + i / kExRX;
        float v = 0.0f;
        uint8_t k = 0;
        if (gx >= 0 && gx < F.w && gy >= 0 && gy < F.h) {
            const size_t g = size_t(gy) * F.w + gx;
            v = F.in[g];
            k = F.in_ok[g];
        }
        s_val[0][i] = v;
        s_ok[0][i] = k;
    }
    __syncthreads();
    // sweep 1 on the region one face inside the staged one (faces outside
    // the field stay invalid)
    for (int j = threadIdx.x; j < (kExRX - 2) * (kExRY - 2); j += blockDim.x) {
        const int rx = 1 + j % (kExRX - 2), ry = 1 + j / (kExRX - 2);
        const int i = ry * kExRX + rx;
        const int gx = x0 + rx, gy = y0 + ry;
        float v = 0.0f;
        uint8_t k = 0;
        if (gx >= 0 && gx < F.w && gy >= 0 && gy < F.h) ex_face(s_val[0], s_ok[0], i, &v, &k);
        s_val[1][i] = v;
        s_ok[1][i] = k;
    }
    __syncthreads();
    // sweep 2 on the tile, written out
    for (int j = threadIdx.x; j < kExTX * kExTY; j += blockDim.x) {
        const int rx = kExHalo + j % kExTX, ry = kExHalo + j / kExTX;
        const int gx = x0 + rx, gy = y0 + ry;
        if (gx >= F.w || gy >= F.h) continue;
        float v;
        uint8_t k;
        ex_face(s_val[1], s_ok[1], ry * kExRX + rx, &v, &k);
        const size_t g = size_t(gy) * F.w + gx;
        F.out[g] = v;
        F.out_ok[g] = k;
    }
}

__global__ void __launch_bounds__(256) k_smoothed_view(uint32_t cells, const float* __restrict__ sm,
                                                       const float* __restrict__ dens,
                                                       const uint32_t* __restrict__ fluid, float* __restrict__ out) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < cells) out[c] = smoothed_at(sm, dens, fluid, c);
}

}  // namespace

uint32_t seg_grid(uint32_t words) {
    uint32_t b = div_up(words, kSegWarps);
    // Levels of up to 2 M cells are latency bound: four CTAs per SM (fewer
    // block partials for the next kernel to sum) beat eight by 2% per PCG
    // iteration at 1024^2; a 4096^2 base level needs every warp slot for
    // bandwidth (eight: 955 vs 1206 us per iteration).
    const uint32_t cap = words <= 65536u ? uint32_t(kMaxRedBlocks) / 2u : uint32_t(kMaxRedBlocks);
    if (b > cap) b = cap;
    return b ? b : 1;
}

cudaError_t launch_finalize_faces(Scene& s, bool forces, bool gravity) {
    uint32_t nf = s.uf + s.vf;
    launch(s.use_pdl, k_faces, div_up(nf, 256), 256, 0, s.stream, s.uf, s.vf, int(s.W), int(s.H), s.acc_u, s.acc_uw, s.acc_v,
                                                    s.acc_vw, s.u, s.v, s.valid_u, s.valid_v, s.ext_u, s.ext_v,
                                                    s.lv[0].fluid, s.obstacle, s.ctl, s.props.gravity, 1,
                                                    forces ? 1 : 0, gravity ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_external_forces(Scene& s) {
    uint32_t nf = s.uf + s.vf;
    launch(s.use_pdl, k_faces, div_up(nf, 256), 256, 0, s.stream, s.uf, s.vf, int(s.W), int(s.H), s.acc_u, s.acc_uw, s.acc_v,
                                                    s.acc_vw, s.u, s.v, s.valid_u, s.valid_v, s.ext_u, s.ext_v,
                                                    s.lv[0].fluid, s.obstacle, s.ctl, s.props.gravity, 0, 1, 1);
    return cudaGetLastError();
}

static cudaError_t compact_level(Scene& s, int level, const uint32_t* obstacle) {
    Level& L = s.lv[level];
    if (level > 0 && L.words <= kOneWords) {
        launch(s.use_pdl, k_compact_one, 1, kOneThreads, 0, s.stream, static_cast<const uint32_t*>(L.fluid), L.words,
               L.seg, level, s.ctl);
        return cudaGetLastError();
    }
    uint32_t nb = div_up(L.words, kCompactWords);
    if (nb == 0) nb = 1;  // the last block records the (empty) level's totals
    launch(s.use_pdl, k_compact_count, nb, 256, 0, s.stream, L.fluid, obstacle, L.words, s.scan_tmp);
    launch(s.use_pdl, k_compact_write, nb, 256, 0, s.stream, static_cast<const uint32_t*>(L.fluid), L.words,
           static_cast<const uint32_t*>(s.scan_tmp), L.seg, L.w, level, s.ctl);
    return cudaGetLastError();
}

cudaError_t launch_base_lists(Scene& s) { return compact_level(s, 0, s.obstacle); }
cudaError_t launch_level_lists(Scene& s, int level) { return compact_level(s, level, nullptr); }

cudaError_t launch_build_pressure(Scene& s) {
    const Level& B = s.lv[0];
    uint32_t g = seg_grid(B.words);
    launch(s.use_pdl, k_smooth_density, g, kSegBlock, 0, s.stream, B.fluid, B.seg, s.ctl, s.W, s.cells, s.density, s.sm_a);
    launch(s.use_pdl, k_smooth_density, g, kSegBlock, 0, s.stream, B.fluid, B.seg, s.ctl, s.W, s.cells, s.sm_a, s.sm_b);
    launch(s.use_pdl, k_smooth_density, g, kSegBlock, 0, s.stream, B.fluid, B.seg, s.ctl, s.W, s.cells, s.sm_b, s.sm_a);
    launch(s.use_pdl, k_laplacian, g, kSegBlock, 0, s.stream, B.fluid, s.obstacle, B.seg, s.ctl, s.W, s.cells, s.dx, s.u, s.v,
                                               s.sm_a, s.density, B.res, B.diag, B.inv_diag, B.px, B.py);
    return cudaGetLastError();
}

// Levels of at most kTailWords mask words (4096 cells: 64^2 and below) are
// built together by one CTA; each larger level by a coarsening launch and
// its segment list.
constexpr uint32_t kTailWords = 128;
cudaError_t launch_multilevel(Scene& s) {
    int l = 1;
    for (; l < s.nlevels && s.lv[l].words > kTailWords; ++l) {
        Level& c = s.lv[l];
        launch(s.use_pdl, k_coarsen, div_up(uint64_t(c.words) * 32, 256), 256, 0, s.stream, s.lv[l - 1], c);
        cudaError_t e = compact_level(s, l, nullptr);
        if (e != cudaSuccess) return e;
    }
    if (l < s.nlevels) {
        TailLevels t;
        t.first = l;
        t.n = s.nlevels;
        for (int k = 0; k < s.nlevels; ++k) t.lv[k] = s.lv[k];
        launch(s.use_pdl, k_coarsen_tail, 1, kOneThreads, 0, s.stream, t, s.ctl);
    }
    return cudaGetLastError();
}

cudaError_t launch_gradient(Scene& s, bool post) {
    uint32_t nf = s.uf + s.vf;
    launch(s.use_pdl, k_gradient, div_up(nf, 256), 256, 0, s.stream, s.uf, s.vf, int(s.W), int(s.H), 1.0f / s.dx, s.u, s.v,
                                                       s.valid_u, s.valid_v, s.lv[0].fluid, s.obstacle, s.pressure,
                                                       s.sm_a, s.density, s.post_u, s.post_v, s.ctl,
                                                       s.p64_valid ? s.p64 : nullptr, 1, post ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_post_forces(Scene& s) {
    uint32_t nf = s.uf + s.vf;
    launch(s.use_pdl, k_gradient, div_up(nf, 256), 256, 0, s.stream, s.uf, s.vf, int(s.W), int(s.H), 1.0f / s.dx, s.u, s.v,
                                                       s.valid_u, s.valid_v, s.lv[0].fluid, s.obstacle, s.pressure,
                                                       s.sm_a, s.density, s.post_u, s.post_v, s.ctl, nullptr,
                                                       0, 1);
    return cudaGetLastError();
}

// The reference's four sweeps as two launches of two sweeps each:
// u, v -> u_alt, v_alt -> u, v (the result ends where the next stages read it).
cudaError_t launch_extrapolate(Scene& s) {
    auto field = [](const float* in, const uint8_t* in_ok, float* out, uint8_t* out_ok, int w, int h) {
        ExField f;
        f.in = in; f.in_ok = in_ok; f.out = out; f.out_ok = out_ok; f.w = w; f.h = h;
        f.tiles_x = int(div_up(uint32_t(w), kExTX));
        return f;
    };
    const int W = int(s.W), H = int(s.H);
    const uint32_t tiles_u = div_up(uint32_t(W + 1), kExTX) * div_up(uint32_t(H), kExTY);
    const uint32_t tiles_v = div_up(uint32_t(W), kExTX) * div_up(uint32_t(H + 1), kExTY);
    launch(s.use_pdl, k_extrapolate2, tiles_u + tiles_v, 256, 0, s.stream,
           field(s.u, s.valid_u, s.u_alt, s.valid_u_alt, W + 1, H), field(s.v, s.valid_v, s.v_alt, s.valid_v_alt, W, H + 1),
           int(tiles_u));
    launch(s.use_pdl, k_extrapolate2, tiles_u + tiles_v, 256, 0, s.stream,
           field(s.u_alt, s.valid_u_alt, s.u, s.valid_u, W + 1, H), field(s.v_alt, s.valid_v_alt, s.v, s.valid_v, W, H + 1),
           int(tiles_u));
    return cudaGetLastError();
}

cudaError_t launch_smoothed_view(Scene& s, float* out) {
    k_smoothed_view<<<div_up(s.cells, 256), 256, 0, s.stream>>>(s.cells, s.sm_a, s.density, s.lv[0].fluid, out);
    return cudaGetLastError();
}

}  // namespace apic
