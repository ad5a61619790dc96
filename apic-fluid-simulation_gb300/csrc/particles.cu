// particles.cu — particle <-> grid transfers on the GPU.
//
//   k_p2g       transfer_particles_to_grid's scatter (src/apic.rs:1237-1426):
//               APIC momentum and weight to the 4 u and 4 v faces, temporal
//               weight w_t (:1246-1248), cell-centred density (:1260-1284) and
//               the fluid bit of the particle's cell (:1358-1360).
//   k_g2p       transfer_grid_to_particles_and_advect (src/apic.rs:2057-2264)
//               over all padded lanes, fused with the max-speed reduction that
//               the next substep's CFL limit needs (get_max_particle_velocity,
//               :2412-2427) and a count of non-finite lanes.
//   k_vmax      stand-alone max speed (after the particle set is written).
//   k_permute   gather of the nine fields by the sorted `val` (:1068-1110).
//
// The reference sums P2G contributions with float CAS loops, so its sums come
// in thread-schedule order.  Here a CTA first sums its particles'
// contributions in shared memory (hardware float atomics) over the window of
// faces and cells they touch, then adds each touched entry to global memory
// once; both levels are likewise order-dependent at the last bit.  Every other result of these kernels is computed lane by lane with the
// reference's operation order.
#include <cuda_runtime.h>

#include <climits>

#include "apic_device.cuh"
#include "apic_internal.h"

namespace apic {
namespace {

// ---- P2G as an ordered gather ------------------------------------------------
//
// The reference adds every chunk's contributions to a face with a CAS loop
// (add_to_mac :296-344, add_to_vec_f32 :347-369): per chunk of 8 slots and per
// stencil corner k (bl, br, tl, tr), the lanes that hit the same face are
// summed in lane order and that group sum is added to the face.  Run on one
// thread, chunk after chunk, a face's sum is therefore the fold of its
// (chunk, corner) group sums in that order, which is the order the oracle
// defines.  Here every face is summed by one thread in exactly that order, so
// the result is bit-identical to the oracle and the same on every run:
//
//   k_p2g_bin_keys  key = the cell of the density stencil's base (cx0, cy0)
//                   for every particle; fluid bits (an OR: order-free)
//   radix sort      stable, so each cell's particles stay in slot order
//   k_p2g_bounds    each cell's run [lo, hi) in the sorted pairs
//   k_p2g_gather    per 32 x 8 tile of cells: stage the particles of the
//                   tile's cells and a two-cell halo below and to the left in
//                   shared memory (in bands of rows when they do not fit),
//                   compute their stencil contributions once per grid, then
//                   let each face merge the runs of the (up to six) cells
//                   whose particles can reach it by slot and fold the
//                   contributions in (chunk, corner, lane) order.
//
// Which cells can reach a face follows from the clamped index arithmetic
// (u_index / v_index, :1029-1041): the u stencil's rows equal the density
// stencil's rows and its columns start at cx0 or cx0 + 1; the v stencil's
// columns equal the density stencil's and its rows start at cy0 or cy0 + 1.
// So u face (i, j) gathers from cells x in [i-2, i], y in [j-1, j], v face
// (i, j) from x in [i-1, i], y in [j-2, j], and density cell (i, j) from
// x in [i-1, i], y in [j-1, j].  A particle whose corners fall outside those
// offsets (impossible by the arithmetic above, checked anyway) raises
// kStatusP2gLayout.
constexpr int kGatherTW = 32, kGatherTH = 8;           // tile of cells, one thread per cell
constexpr int kGatherThreads = kGatherTW * kGatherTH;
constexpr int kRegionW = kGatherTW + 2, kRegionH = kGatherTH + 2;
constexpr int kRegionBins = kRegionW * kRegionH;       // 340 cells whose particles a tile reads
constexpr int kGatherCap = 2048;                       // staged particles per tile (more: read from global)
// slot, corner code, 4 values, 4 weights, and the grid position and temporal
// weight that every grid's contributions share
constexpr size_t kGatherSmem = size_t(kGatherCap) * (4 + 4 + 8 * 4 + 3 * 4) + size_t(kRegionBins) * 8 + 64;

enum { kGridU = 0, kGridV = 1, kGridD = 2 };

// Exclusive scan over the threads of a block (blockDim.x a multiple of 32).
__device__ __forceinline__ uint32_t block_exclusive_scan_u32(uint32_t v, uint32_t* total) {
    __shared__ uint32_t sw[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sw[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = lane < int(blockDim.x / 32) ? sw[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        sw[lane] = t;
    }
    __syncthreads();
    const uint32_t pre = warp > 0 ? sw[warp - 1] : 0u;
    *total = sw[blockDim.x / 32 - 1];
    __syncthreads();
    return pre + x - v;
}

// Four particles per thread with 16-byte loads and stores (the arrays hold
// npad, a multiple of 8, lanes; keys of lanes n .. npad-1 are never read).
__global__ void __launch_bounds__(256) k_p2g_bin_keys(const PartPtrs* __restrict__ pp, uint32_t n, int W, int H,
                                                      float dx, uint32_t* __restrict__ keys,
                                                      uint32_t* __restrict__ vals, uint32_t* __restrict__ fluid) {
    pdl_wait();
    const uint32_t i0 = 4u * (blockIdx.x * blockDim.x + threadIdx.x);
    const bool any = i0 < n;
    float4 px = make_float4(0.0f, 0.0f, 0.0f, 0.0f), py = px;
    if (any) {
        px = *reinterpret_cast<const float4*>(pp->f[PX] + i0);
        py = *reinterpret_cast<const float4*>(pp->f[PY] + i0);
    }
    const float xs[4] = {px.x, px.y, px.z, px.w}, ys[4] = {py.x, py.y, py.z, py.w};
    uint32_t k[4];
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const bool live = i0 + uint32_t(q) < n;
        const float gx = xs[q] / dx, gy = ys[q] / dx;
        const int cx0 = max(min(trunc_x86(floorf(gx - 0.5f)), W - 1), 0);
        const int cy0 = max(min(trunc_x86(floorf(gy - 0.5f)), H - 1), 0);
        k[q] = uint32_t(cy0) * uint32_t(W) + uint32_t(cx0);
        // the particle's own cell (:1358-1360); one OR per mask word the warp touches
        const int fx = trunc_x86(fmax_x86(fmin_x86(gx, float(W) - 1.0f), 0.0f));
        const int fy = trunc_x86(fmax_x86(fmin_x86(gy, float(H) - 1.0f), 0.0f));
        const uint32_t fi = uint32_t(fy * W + fx);
        const uint32_t word = live ? fi >> 5 : 0xFFFFFFFFu, bit = live ? 1u << (fi & 31u) : 0u;
        const uint32_t peers = __match_any_sync(0xffffffffu, word);
        const uint32_t m = __reduce_or_sync(peers, bit);
        if (live && (peers & ((1u << lane) - 1u)) == 0) atomicOr(fluid + word, m);
    }
    if (any) {
        *reinterpret_cast<uint4*>(keys + i0) = make_uint4(k[0], k[1], k[2], k[3]);
        *reinterpret_cast<uint4*>(vals + i0) = make_uint4(i0, i0 + 1, i0 + 2, i0 + 3);
    }
}

__global__ void __launch_bounds__(256) k_p2g_bounds(const uint32_t* __restrict__ keys, uint32_t n,
                                                    uint32_t* __restrict__ lo, uint32_t* __restrict__ hi,
                                                    uint32_t cells, uint32_t* __restrict__ status) {
    pdl_wait();
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t k = keys[j];
    if (!APIC_IN_BOUNDS(k, cells, status)) return;
    if (j == 0 || keys[j - 1] != k) lo[k] = j;
    if (j == n - 1 || keys[j + 1] != k) hi[k] = j + 1;
}

// One particle's contributions to one grid: per corner k the value and weight
// (value unused for the density) and, per relative face position q of the
// face that gathers it (q = ry * nx + rx, offsets from the particle's density
// base cell), a 4-bit mask of the corners that land there.
struct P2gRec {
    uint32_t code;
    float val[4], w[4];
};

// The quantities of one particle that every grid's contributions share:
// grid position and temporal weight (:1246-1256).
struct P2gBase {
    float gx, gy, wt;
};
__device__ __forceinline__ P2gBase p2g_base(const PartPtrs* __restrict__ pp, uint32_t slot, float dx, float prev_dt) {
    const float tr = pp->f[TR][slot];
    const float tau = (-tr) / prev_dt;
    P2gBase b;
    b.wt = temporal_w(tau);
    b.gx = pp->f[PX][slot] / dx;
    b.gy = pp->f[PY][slot] / dx;
    return b;
}

__device__ __forceinline__ bool p2g_record(const PartPtrs* __restrict__ pp, uint32_t slot, const P2gBase& b, int grid,
                                           int W, int H, float dx, P2gRec& r) {
    const float gx = b.gx, gy = b.gy, wt = b.wt;
    const int cx0 = max(min(trunc_x86(floorf(gx - 0.5f)), W - 1), 0);
    const int cy0 = max(min(trunc_x86(floorf(gy - 0.5f)), H - 1), 0);
    int xs[2], ys[2], nx, ny;
    if (grid == kGridD) {
        // cell-centred density stencil (:1260-1284)
        const float cgx = gx - 0.5f, cgy = gy - 0.5f;
        const float cbx = floorf(cgx), cby = floorf(cgy);
        const float ctx = cgx - cbx, cty = cgy - cby;
        r.w[0] = ((1.0f - ctx) * (1.0f - cty)) * wt;
        r.w[1] = (ctx * (1.0f - cty)) * wt;
        r.w[2] = ((1.0f - ctx) * cty) * wt;
        r.w[3] = (ctx * cty) * wt;
        const int tbx = trunc_x86(cbx), tby = trunc_x86(cby);
        xs[0] = max(min(tbx, W - 1), 0); xs[1] = max(min(tbx + 1, W - 1), 0);
        ys[0] = max(min(tby, H - 1), 0); ys[1] = max(min(tby + 1, H - 1), 0);
        nx = 2; ny = 2;
    } else if (grid == kGridU) {
        Stencil su;
        u_stencil(gx, gy, W, H, dx, su);
        const float vx = pp->f[VX][slot], cux = pp->f[CUX][slot], cuy = pp->f[CUY][slot];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            r.w[k] = su.w[k] * wt;
            r.val[k] = (vx + cux * su.ox[k] + cuy * su.oy[k]) * r.w[k];
        }
        const int ix = trunc_x86(floorf(gx)), iy = trunc_x86(floorf(gy - 0.5f));
        xs[0] = max(min(ix, W), 0); xs[1] = max(min(ix + 1, W), 0);
        ys[0] = max(min(iy, H - 1), 0); ys[1] = max(min(iy + 1, H - 1), 0);
        nx = 3; ny = 2;
    } else {
        Stencil sv;
        v_stencil(gx, gy, W, H, dx, sv);
        const float vy = pp->f[VY][slot], cvx = pp->f[CVX][slot], cvy = pp->f[CVY][slot];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            r.w[k] = sv.w[k] * wt;
            r.val[k] = (vy + cvx * sv.ox[k] + cvy * sv.oy[k]) * r.w[k];
        }
        const int jx = trunc_x86(floorf(gx - 0.5f)), jy = trunc_x86(floorf(gy));
        xs[0] = max(min(jx, W - 1), 0); xs[1] = max(min(jx + 1, W - 1), 0);
        ys[0] = max(min(jy, H), 0); ys[1] = max(min(jy + 1, H), 0);
        nx = 2; ny = 3;
    }
    uint32_t code = 0;
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int rx = xs[k & 1] - cx0, ry = ys[k >> 1] - cy0;
        if (rx < 0 || rx >= nx || ry < 0 || ry >= ny) {
            ok = false;
            continue;
        }
        code |= (1u << k) << (4 * (ry * nx + rx));
    }
    r.code = code;
    return ok;
}

// Records staged in shared memory (fast path) or computed from global memory
// when they are needed (regions with more particles than the stage holds).
// A staged slot carries kLastInRun in bit 31 when it is the last particle of
// its cell's run (slots are below 2^31).
constexpr uint32_t kLastInRun = 0x80000000u;
struct StagedRecs {
    static constexpr bool kStaged = true;
    const uint32_t* slot;
    const uint32_t* code;
    const float* val;  // [4][kGatherCap]
    const float* w;    // [4][kGatherCap]
    __device__ __forceinline__ uint32_t code_at(int p) const { return code[p]; }
    __device__ __forceinline__ float val_at(int k, int p) const { return val[k * kGatherCap + p]; }
    __device__ __forceinline__ float w_at(int k, int p) const { return w[k * kGatherCap + p]; }
};
struct GlobalRecs {
    static constexpr bool kStaged = false;
    const uint32_t* vals;  // sorted slots
    const PartPtrs* pp;
    int grid, W, H;
    float dx, prev_dt;
    uint32_t* status;
    uint32_t n, npad;  // sorted pairs, particle lanes (the checked build tests against them)
    __device__ __forceinline__ uint32_t slot_at(int p) const {
        const uint32_t sl = APIC_IN_BOUNDS(uint32_t(p), n, status) ? vals[p] : 0u;
        return APIC_IN_BOUNDS(sl, npad, status) ? sl : 0u;
    }
    __device__ __forceinline__ P2gRec rec(int p) const {
        P2gRec r;
        const uint32_t sl = slot_at(p);
        if (!p2g_record(pp, sl, p2g_base(pp, sl, dx, prev_dt), grid, W, H, dx, r)) atomicOr(status, kStatusP2gLayout);
        return r;
    }
    __device__ __forceinline__ uint32_t code_at(int p) const { return rec(p).code; }
    __device__ __forceinline__ float val_at(int k, int p) const { return rec(p).val[k]; }
    __device__ __forceinline__ float w_at(int k, int p) const { return rec(p).w[k]; }
};

// The fold of one face over its contributions in slot order.  Consecutive
// contributions of one chunk form the chunk's groups: per corner k, the
// lanes' contributions summed in lane order; at the end of the chunk the
// groups are added to the face in corner order.
struct FaceFold {
    float acc_v = 0.0f, acc_w = 0.0f;
    float gv[4] = {0.0f, 0.0f, 0.0f, 0.0f}, gw[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    uint32_t gm = 0, chunk = 0xFFFFFFFFu;
    template <bool kVal, class Recs>
    __device__ __forceinline__ void add(const Recs& R, uint32_t slot, int p, uint32_t hit) {
        if ((slot >> 3) != chunk) {
            flush<kVal>();
            chunk = slot >> 3;
        }
        // only the corners that land here are read (usually one)
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (hit & (1u << k)) {
                if (kVal) gv[k] = gv[k] + R.val_at(k, p);
                gw[k] = gw[k] + R.w_at(k, p);
            }
        gm |= hit;
    }
    template <bool kVal>
    __device__ __forceinline__ void flush() {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (gm & (1u << k)) {
                if (kVal) acc_v = acc_v + gv[k];
                acc_w = acc_w + gw[k];
            }
#pragma unroll
        for (int k = 0; k < 4; ++k) { gv[k] = 0.0f; gw[k] = 0.0f; }
        gm = 0;
    }
};

// Fold of one face: merge NR slot-ordered runs [b, e) by slot; run r's
// records reach this face through the corners in bits 4r .. 4r + 3 of their
// code.
//
// Staged form: each run's head is one 64-bit key (slot << 32 | position << 5
// | last-in-run << 4 | run), so the merge step is a minimum over NR keys and
// the head's successor is the next staged position unless the head ends its
// run.  Global form: positions and ends in registers.
template <int NR, bool kVal, bool kRef, class Recs>
__device__ __forceinline__ void fold_face(const Recs& R, int (&b)[NR], const int (&e)[NR], float& out_v,
                                          float& out_w) {
    if constexpr (!kRef) {
        // cell order: the runs one after another, slots ascending in each,
        // the corners that land here in corner order
        float av = 0.0f, aw = 0.0f;
#pragma unroll
        for (int r = 0; r < NR; ++r)
            for (int p = b[r]; p < e[r]; ++p) {
                if constexpr (Recs::kStaged) {
                    const uint32_t hit = (R.code_at(p) >> (4 * r)) & 0xFu;
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (hit & (1u << k)) {
                            if (kVal) av = av + R.val_at(k, p);
                            aw = aw + R.w_at(k, p);
                        }
                } else {
                    const P2gRec rr = R.rec(p);
                    const uint32_t hit = (rr.code >> (4 * r)) & 0xFu;
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (hit & (1u << k)) {
                            if (kVal) av = av + rr.val[k];
                            aw = aw + rr.w[k];
                        }
                }
            }
        out_v = av;
        out_w = aw;
        return;
    }
    FaceFold f;
    if constexpr (Recs::kStaged) {
        auto key_at = [&](uint32_t p, uint32_t r) {
            const uint32_t sw = R.slot[p];
            return (uint64_t(sw & ~kLastInRun) << 32) | (uint64_t(p) << 5) | (uint64_t(sw >> 31) << 4) | uint64_t(r);
        };
        uint64_t key[NR];
#pragma unroll
        for (int r = 0; r < NR; ++r) key[r] = b[r] < e[r] ? key_at(uint32_t(b[r]), uint32_t(r)) : ~0ull;
        for (;;) {
            uint64_t best = key[0];
#pragma unroll
            for (int r = 1; r < NR; ++r) best = key[r] < best ? key[r] : best;
            if (best == ~0ull) break;
            const uint32_t m = uint32_t(best) & 0xFu;
            const uint32_t p = uint32_t(best >> 5) & 0x07FFFFFFu;
            const uint64_t nk = ((best >> 4) & 1u) ? ~0ull : key_at(p + 1u, m);
#pragma unroll
            for (int r = 0; r < NR; ++r) key[r] = uint32_t(r) == m ? nk : key[r];
            const uint32_t hit = (R.code_at(int(p)) >> (4u * m)) & 0xFu;
            if (hit) f.template add<kVal>(R, uint32_t(best >> 32), int(p), hit);
        }
    } else {
        uint32_t hs[NR];
#pragma unroll
        for (int r = 0; r < NR; ++r) hs[r] = b[r] < e[r] ? R.slot_at(b[r]) : 0xFFFFFFFFu;
        for (;;) {
            uint32_t best = hs[0];
            int m = 0;
#pragma unroll
            for (int r = 1; r < NR; ++r)
                if (hs[r] < best) { best = hs[r]; m = r; }
            if (best == 0xFFFFFFFFu) break;
            int p = 0;
#pragma unroll
            for (int r = 0; r < NR; ++r)
                if (r == m) {
                    p = b[r];
                    b[r] = p + 1;
                    hs[r] = b[r] < e[r] ? R.slot_at(b[r]) : 0xFFFFFFFFu;
                }
            const uint32_t hit = (R.code_at(p) >> (4 * m)) & 0xFu;
            if (hit) f.template add<kVal>(R, best, p, hit);
        }
    }
    f.template flush<kVal>();
    out_v = f.acc_v;
    out_w = f.acc_w;
}

struct GatherOut {
    float *acc_u, *acc_uw, *acc_v, *acc_vw, *dens;
};

// The faces and cells of this thread's cell (i, j) for one grid; bin(x, y)
// gives a cell's run (empty outside the grid).  Run r of a face is the cell
// at offset (rx, ry) with r = ry * nx + rx, the index p2g_record codes.
template <bool kRef, class Recs, class Bin>
__device__ __forceinline__ void fold_cell(const Recs& R, const Bin& bin, int grid, int i, int j, int W, int H,
                                          const GatherOut& o) {
    auto run = [&](int x, int y, int& b, int& e) {
        if (x < 0 || x >= W || y < 0 || y >= H) { b = e = 0; return; }
        bin(x, y, b, e);
    };
    if (grid == kGridU) {
        // u face (fi, j), and (W, j) from the last column's thread
        for (int fi = i; fi <= (i == W - 1 ? W : i); ++fi) {
            int b[6], e[6];
#pragma unroll
            for (int r = 0; r < 6; ++r) run(fi - r % 3, j - r / 3, b[r], e[r]);
            float v, w;
            fold_face<6, true, kRef>(R, b, e, v, w);
            const uint32_t f = uint32_t(j) * uint32_t(W + 1) + uint32_t(fi);
            o.acc_u[f] = v;
            o.acc_uw[f] = w;
        }
    } else if (grid == kGridV) {
        for (int fj = j; fj <= (j == H - 1 ? H : j); ++fj) {
            int b[6], e[6];
#pragma unroll
            for (int r = 0; r < 6; ++r) run(i - r % 2, fj - r / 2, b[r], e[r]);
            float v, w;
            fold_face<6, true, kRef>(R, b, e, v, w);
            const uint32_t f = uint32_t(fj) * uint32_t(W) + uint32_t(i);
            o.acc_v[f] = v;
            o.acc_vw[f] = w;
        }
    } else {
        int b[4], e[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) run(i - r % 2, j - r / 2, b[r], e[r]);
        float v, w;
        fold_face<4, false, kRef>(R, b, e, v, w);
        o.dens[uint32_t(j) * uint32_t(W) + uint32_t(i)] = w;
    }
}

// One CTA per 32 x 8 tile.  The region's cell counts are scanned once; when
// the region holds more particles than the stage (dense scenes: the
// reference's default block has 9 per cell), the tile is processed as 2, 4
// or 8 bands of rows, each staging only its own region (band rows plus the
// two-row halo); a single row whose region still overflows reads its records
// from global memory.  kRef: the reference's order, else cell order
// (APIC_OPT_P2G_ORDER).
template <bool kRef>
__global__ void __launch_bounds__(kGatherThreads, 2) k_p2g_gather(const PartPtrs* __restrict__ pp,
                                                                  const uint32_t* __restrict__ vals,
                                                                  const uint32_t* __restrict__ lo,
                                                                  const uint32_t* __restrict__ hi, int W, int H,
                                                                  float dx, Ctl* __restrict__ ctl, GatherOut o,
                                                                  uint32_t n, uint32_t npad) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* s_slot = reinterpret_cast<uint32_t*>(smem);
    uint32_t* s_code = s_slot + kGatherCap;
    float* s_val = reinterpret_cast<float*>(s_code + kGatherCap);
    float* s_w = s_val + 4 * kGatherCap;
    float* s_gx = s_w + 4 * kGatherCap;
    float* s_gy = s_gx + kGatherCap;
    float* s_wt = s_gy + kGatherCap;
    uint32_t* s_off = reinterpret_cast<uint32_t*>(s_wt + kGatherCap);  // kRegionBins + 1
    uint32_t* s_glo = s_off + kRegionBins + 1;                            // kRegionBins
    __shared__ uint32_t s_total, s_band;
    __shared__ uint32_t s_rowg[kRegionH];

    const int x0 = blockIdx.x * kGatherTW, y0 = blockIdx.y * kGatherTH;
    const int rx0 = x0 - 2, ry0 = y0 - 2;
    const int tx = threadIdx.x % kGatherTW, ty = threadIdx.x / kGatherTW;
    const int i = x0 + tx, j = y0 + ty;
    const bool cell = i < W && j < H;
    pdl_wait();
    const float prev_dt = ctl->prev_dt;

    // the region's runs: counts, their exclusive scan, first global position per row
    if (threadIdx.x < kRegionH) s_rowg[threadIdx.x] = 0xFFFFFFFFu;
    uint32_t cnt[2] = {0u, 0u};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int rb = 2 * threadIdx.x + h;
        if (rb < kRegionBins) {
            const int x = rx0 + rb % kRegionW, y = ry0 + rb / kRegionW;
            uint32_t gl = 0, gh = 0;
            if (x >= 0 && x < W && y >= 0 && y < H) {
                const uint32_t c = uint32_t(y) * uint32_t(W) + uint32_t(x);
                gl = lo[c];
                gh = hi[c];
            }
            cnt[h] = gh - gl;
            s_glo[rb] = gl;
        }
    }
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan_u32(cnt[0] + cnt[1], &tot);
    if (2 * threadIdx.x < kRegionBins) s_off[2 * threadIdx.x] = ex;
    if (2 * threadIdx.x + 1 < kRegionBins) s_off[2 * threadIdx.x + 1] = ex + cnt[0];
    if (threadIdx.x == 0) { s_off[kRegionBins] = tot; s_total = tot; }
    __syncthreads();
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int rb = 2 * threadIdx.x + h;
        if (rb < kRegionBins && cnt[h] > 0) atomicMin(&s_rowg[rb / kRegionW], s_glo[rb]);
    }
    if (threadIdx.x == 0) {
        // the tallest band whose every region fits the stage (0: none)
        uint32_t band = 0;
        for (uint32_t th = kGatherTH; th >= 1 && !band; th >>= 1) {
            bool fits = true;
            for (uint32_t r0 = 0; r0 < uint32_t(kGatherTH); r0 += th)
                fits = fits && s_off[(r0 + th + 2) * kRegionW] - s_off[r0 * kRegionW] <= uint32_t(kGatherCap);
            if (fits) band = th;
        }
        s_band = band;
    }
    __syncthreads();
    const uint32_t band = s_band;

    if (band == 0) {
        // more particles than the stage holds even for one row: every face
        // reads its runs from global memory and computes the records it needs
        for (int g = 0; g < 3; ++g) {
            GlobalRecs R{vals, pp, g, W, H, dx, prev_dt, &ctl->status, n, npad};
            auto bin = [&](int x, int y, int& b, int& e) {
                const uint32_t c = uint32_t(y) * uint32_t(W) + uint32_t(x);
                b = int(lo[c]);
                e = int(hi[c]);
            };
            if (cell) fold_cell<kRef>(R, bin, g, i, j, W, H, o);
        }
        return;
    }
    const StagedRecs R{s_slot, s_code, s_val, s_w};
    for (uint32_t r0 = 0; r0 < uint32_t(kGatherTH); r0 += band) {
        const uint32_t r1 = r0 + band + 2;  // region rows [r0, r1)
        const uint32_t base = s_off[r0 * kRegionW];
        const uint32_t P = s_off[r1 * kRegionW] - base;
        // stage the slots: each region row is one contiguous range of the sorted pairs
        for (uint32_t r = r0; r < r1; ++r) {
            const uint32_t s0 = s_off[r * kRegionW] - base, s1 = s_off[(r + 1) * kRegionW] - base;
            const uint32_t g0 = s_rowg[r];
            for (uint32_t q = threadIdx.x; q < s1 - s0; q += kGatherThreads) {
                const uint32_t sl = APIC_IN_BOUNDS(g0 + q, n, &ctl->status) ? vals[g0 + q] : 0u;
                s_slot[s0 + q] = APIC_IN_BOUNDS(sl, npad, &ctl->status) ? sl : 0u;
            }
        }
        __syncthreads();
        if constexpr (kRef) {
            // mark each run's last particle (the merge reads it)
            for (uint32_t rb = r0 * kRegionW + threadIdx.x; rb < r1 * kRegionW; rb += kGatherThreads)
                if (s_off[rb + 1] > s_off[rb]) s_slot[s_off[rb + 1] - 1u - base] |= kLastInRun;
            __syncthreads();
        }
        for (uint32_t p = threadIdx.x; p < P; p += kGatherThreads) {
            const P2gBase bs = p2g_base(pp, s_slot[p] & ~kLastInRun, dx, prev_dt);
            s_gx[p] = bs.gx;
            s_gy[p] = bs.gy;
            s_wt[p] = bs.wt;
        }
        auto bin = [&](int x, int y, int& b, int& e) {
            const int rb = (y - ry0) * kRegionW + (x - rx0);
            b = int(s_off[rb] - base);
            e = int(s_off[rb + 1] - base);
        };
        const bool mine = cell && uint32_t(ty) >= r0 && uint32_t(ty) < r0 + band;
        for (int g = 0; g < 3; ++g) {
            bool bad = false;
            for (uint32_t p = threadIdx.x; p < P; p += kGatherThreads) {
                P2gRec rec;
                const P2gBase bs{s_gx[p], s_gy[p], s_wt[p]};
                if (!p2g_record(pp, s_slot[p] & ~kLastInRun, bs, g, W, H, dx, rec)) bad = true;
                s_code[p] = rec.code;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (g != kGridD) s_val[k * kGatherCap + p] = rec.val[k];
                    s_w[k * kGatherCap + p] = rec.w[k];
                }
            }
            if (bad) atomicOr(&ctl->status, kStatusP2gLayout);
            __syncthreads();
            if (mine) fold_cell<kRef>(R, bin, g, i, j, W, H, o);
            __syncthreads();
        }
    }
}

// Cell order (APIC_OPT_P2G_ORDER 2), one CTA per 32 x 8 tile.  Each cell of
// the tile's region (the tile plus two halo columns on the left and two halo
// rows below) is summed by one thread: its particles in slot order, each
// particle's corners in corner order, into one partial sum per relative face
// position (6 u, 6 v, 4 density positions; the code bits of p2g_record).
// Each face then adds the partial sums of the cells that reach it in run
// order (the reference-order gather's cell offsets); empty cells are
// skipped.  The terms are those of the reference's order; only the
// association differs.  No particle is staged, so dense cells need no
// fallback.
constexpr int kCellRegion = kRegionW * kRegionH;  // 340
struct CellPartials {
    float uv[6][kCellRegion], uw[6][kCellRegion];
    float vv[6][kCellRegion], vw[6][kCellRegion];
    float dw[4][kCellRegion];
    uint8_t has[kCellRegion];
};

template <int NQ, bool kVal>
__device__ __forceinline__ void add_partials(const P2gRec& rec, float (&pv)[NQ], float (&pw)[NQ]) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        const uint32_t hit = (rec.code >> (4 * q)) & 0xFu;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (hit & (1u << k)) {
                if (kVal) pv[q] = pv[q] + rec.val[k];
                pw[q] = pw[q] + rec.w[k];
            }
    }
}

// One thread per region cell (352 threads for 340 cells, then the tile's 256
// cells' faces), two CTAs per SM: the per-cell loops are load-latency bound.
constexpr int kCellThreads = 352;
// kMinB 3 (56 registers, some spilled) for grids of more than 2 M cells
// (4096^2: 3.56 vs 3.79 ms per P2G stage), 2 below.
template <int kMinB>
__global__ void __launch_bounds__(kCellThreads, kMinB) k_p2g_cells(const PartPtrs* __restrict__ pp,
                                                                 const uint32_t* __restrict__ vals,
                                                                 const uint32_t* __restrict__ lo,
                                                                 const uint32_t* __restrict__ hi, int W, int H,
                                                                 float dx, Ctl* __restrict__ ctl, GatherOut o,
                                                                 uint32_t n, uint32_t npad) {
    __shared__ CellPartials sp;
    const int x0 = blockIdx.x * kGatherTW, y0 = blockIdx.y * kGatherTH;
    const int rx0 = x0 - 2, ry0 = y0 - 2;
    pdl_wait();
    const float prev_dt = ctl->prev_dt;
    bool bad = false;
    for (int rc = threadIdx.x; rc < kCellRegion; rc += kCellThreads) {
        const int x = rx0 + rc % kRegionW, y = ry0 + rc / kRegionW;
        uint32_t b = 0, e = 0;
        if (x >= 0 && x < W && y >= 0 && y < H) {
            const uint32_t c = uint32_t(y) * uint32_t(W) + uint32_t(x);
            b = lo[c];
            e = hi[c];
        }
        float uv[6] = {}, uw[6] = {}, vv[6] = {}, vw[6] = {}, dv[4] = {}, dw[4] = {};
        // the next particle's slot is loaded while this one's fields are
        if (!APIC_IN_BOUNDS(e, uint64_t(n) + 1u, &ctl->status)) e = b;
        uint32_t next = b < e ? vals[b] : 0u;
        for (uint32_t p = b; p < e; ++p) {
            const uint32_t slot = next;
            if (p + 1 < e) next = vals[p + 1];
            if (!APIC_IN_BOUNDS(slot, npad, &ctl->status)) continue;
            const P2gBase bs = p2g_base(pp, slot, dx, prev_dt);
            P2gRec rec;
            if (!p2g_record(pp, slot, bs, kGridU, W, H, dx, rec)) bad = true;
            add_partials<6, true>(rec, uv, uw);
            if (!p2g_record(pp, slot, bs, kGridV, W, H, dx, rec)) bad = true;
            add_partials<6, true>(rec, vv, vw);
            if (!p2g_record(pp, slot, bs, kGridD, W, H, dx, rec)) bad = true;
            add_partials<4, false>(rec, dv, dw);
        }
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            sp.uv[q][rc] = uv[q];
            sp.uw[q][rc] = uw[q];
            sp.vv[q][rc] = vv[q];
            sp.vw[q][rc] = vw[q];
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) sp.dw[q][rc] = dw[q];
        sp.has[rc] = e > b;
    }
    if (bad) atomicOr(&ctl->status, kStatusP2gLayout);
    __syncthreads();
    if (threadIdx.x >= kGatherThreads) return;
    const int tx = threadIdx.x % kGatherTW, ty = threadIdx.x / kGatherTW;
    const int i = x0 + tx, j = y0 + ty;
    if (i >= W || j >= H) return;
    // region index of cell (x, y), or -1 when it holds no particle (or lies
    // outside the grid)
    auto cell = [&](int x, int y) -> int {
        if (x < 0 || y < 0 || x >= W || y >= H) return -1;
        const int rc = (y - ry0) * kRegionW + (x - rx0);
        return sp.has[rc] ? rc : -1;
    };
    for (int fi = i; fi <= (i == W - 1 ? W : i); ++fi) {
        float av = 0.0f, aw = 0.0f;
#pragma unroll
        for (int r = 0; r < 6; ++r) {
            const int rc = cell(fi - r % 3, j - r / 3);
            if (rc >= 0) {
                av = av + sp.uv[r][rc];
                aw = aw + sp.uw[r][rc];
            }
        }
        const uint32_t f = uint32_t(j) * uint32_t(W + 1) + uint32_t(fi);
        o.acc_u[f] = av;
        o.acc_uw[f] = aw;
    }
    for (int fj = j; fj <= (j == H - 1 ? H : j); ++fj) {
        float av = 0.0f, aw = 0.0f;
#pragma unroll
        for (int r = 0; r < 6; ++r) {
            const int rc = cell(i - r % 2, fj - r / 2);
            if (rc >= 0) {
                av = av + sp.vv[r][rc];
                aw = aw + sp.vw[r][rc];
            }
        }
        const uint32_t f = uint32_t(fj) * uint32_t(W) + uint32_t(i);
        o.acc_v[f] = av;
        o.acc_vw[f] = aw;
    }
    float aw = 0.0f;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int rc = cell(i - r % 2, j - r / 2);
        if (rc >= 0) aw = aw + sp.dw[r][rc];
    }
    o.dens[uint32_t(j) * uint32_t(W) + uint32_t(i)] = aw;
}

// bilinear_interpolate, src/apic.rs:138-172.
__device__ __forceinline__ float bilinear(const float w[4], const float v[4]) {
    float ws = w[0] + w[1] + w[2] + w[3];
    float inv = 1.0f / fmax_x86(ws, 1e-6f);
    float vel = 0.0f;
#pragma unroll
    for (int k = 0; k < 4; ++k) vel += v[k] * w[k] * inv;
    return vel;
}

__device__ __forceinline__ void block_max_count(float m, uint32_t bad, Ctl* ctl) {
    __shared__ float sm[8];
    __shared__ uint32_t sb[8];
    m = warp_maxf(m);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) bad += __shfl_xor_sync(0xffffffffu, bad, o);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { sm[warp] = m; sb[warp] = bad; }
    __syncthreads();
    if (threadIdx.x == 0) {
        float bm = 0.0f;
        uint32_t bb = 0;
        for (int w = 0; w < int(blockDim.x / 32); ++w) { bm = fmaxf(bm, sm[w]); bb += sb[w]; }
        if (bm > 0.0f) atomicMax(&ctl->vmax_bits, __float_as_uint(bm));
        if (bb) atomicAdd(&ctl->nonfinite, bb);
    }
}

// four CTAs per SM (64 registers): G2P is bound by the latency of its
// dependent loads (particle, then the faces it gathers); at 4096^2 four CTAs
// per SM take the stage from 0.88 to 0.73 ms
__global__ void __launch_bounds__(256, 4) k_g2p(const PartPtrs* __restrict__ pp, uint32_t npad, int W, int H, float dx,
                                             float border_damping, Ctl* __restrict__ ctl,
                                             const float* __restrict__ gu, const float* __restrict__ gv,
                                             const uint32_t* __restrict__ u_open,
                                             const uint32_t* __restrict__ v_open) {
    pdl_wait();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float speed_out = 0.0f;
    uint32_t bad = 0;
    if (i < npad) {
        const float dt = ctl->dt;
        const uint32_t ts = ctl->timestamp;
        const float min_x = 1.001f * dx, max_x = (float(W) - 1.001f) * dx;
        const float min_y = 1.001f * dx, max_y = (float(H) - 1.001f) * dx;
        const float h2 = dx * dx, eps = 1e-6f, bd = -border_damping;
        float px = pp->f[PX][i], py = pp->f[PY][i];
        float gx = px / dx, gy = py / dx;
        Stencil su, sv;
        u_stencil(gx, gy, W, H, dx, su);
        v_stencil(gx, gy, W, H, dx, sv);
        float un[4], vn[4], uwm[4], vwm[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const bool uin = APIC_IN_BOUNDS(su.idx[k], uint32_t(W + 1) * uint32_t(H), &ctl->status);
            const bool vin = APIC_IN_BOUNDS(sv.idx[k], uint32_t(W) * uint32_t(H + 1), &ctl->status);
            un[k] = uin ? gu[su.idx[k]] : 0.0f;
            vn[k] = vin ? gv[sv.idx[k]] : 0.0f;
            uwm[k] = uin && bit_at(u_open, su.idx[k]) ? su.w[k] : 0.0f;
            vwm[k] = vin && bit_at(v_open, sv.idx[k]) ? sv.w[k] : 0.0f;
        }
        float nvx = bilinear(uwm, un), nvy = bilinear(vwm, vn);
        float res = pp->f[TR][i];
        float speed = sqrtf(nvx * nvx + nvy * nvy);
        float cfl_local = speed * dt / dx;
        float scale = fmin_x86(fmax_x86(cfl_local, 0.0f), 1.0f);
        float gam = scale * scale * (3.0f - (2.0f * scale));
        float jitter = gam * random_lane(i, ts) * dt;
        float dt_raw = dt + res + jitter;
        float dt_act = fmin_x86(fmax_x86(dt_raw, 0.0f), dt * 2.0f);
        float nres = dt + res - dt_act;
        float nx = px + dt_act * nvx, ny = py + dt_act * nvy;
        bool oxmin = nx < min_x, oxmax = nx > max_x, oymin = ny < min_y, oymax = ny > max_y;
        bool ovxmin = oxmin && nvx < 0.0f, ovxmax = oxmax && nvx > 0.0f;
        bool ovymin = oymin && nvy < 0.0f, ovymax = oymax && nvy > 0.0f;
        if (oxmin) nx = min_x;
        if (oxmax) nx = max_x;
        if (ovxmin) nvx = nvx * bd;
        if (ovxmax) nvx = nvx * bd;
        if (oymin) ny = min_y;
        if (oymax) ny = max_y;
        if (ovymin) nvy = nvy * bd;
        if (ovymax) nvy = nvy * bd;
        float udx = h2 * su.tx * (1.0f - su.tx), udy = h2 * su.ty * (1.0f - su.ty);
        float vdx = h2 * sv.tx * (1.0f - sv.tx), vdy = h2 * sv.ty * (1.0f - sv.ty);
        float uix = udx > eps ? 1.0f / udx : 0.0f, uiy = udy > eps ? 1.0f / udy : 0.0f;
        float vix = vdx > eps ? 1.0f / vdx : 0.0f, viy = vdy > eps ? 1.0f / vdy : 0.0f;
        float cux = 0.0f, cuy = 0.0f, cvx = 0.0f, cvy = 0.0f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            cux += su.w[k] * un[k] * su.ox[k];
            cuy += su.w[k] * un[k] * su.oy[k];
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            cvx += sv.w[k] * vn[k] * sv.ox[k];
            cvy += sv.w[k] * vn[k] * sv.oy[k];
        }
        float cu_x = cux * uix, cu_y = cuy * uiy, cv_x = cvx * vix, cv_y = cvy * viy;
        bool rx = ovxmin || ovxmax, ry = ovymin || ovymax;
        if (rx) { cu_y = cu_y * -1.0f; cv_x = cv_x * -1.0f; }
        if (ry) { cu_y = cu_y * -1.0f; cv_x = cv_x * -1.0f; }
        pp->f[PX][i] = nx;
        pp->f[PY][i] = ny;
        pp->f[VX][i] = nvx;
        pp->f[VY][i] = nvy;
        pp->f[CUX][i] = cu_x;
        pp->f[CUY][i] = cu_y;
        pp->f[CVX][i] = cv_x;
        pp->f[CVY][i] = cv_y;
        pp->f[TR][i] = nres;
        float m = sqrtf(nvx * nvx + nvy * nvy);  // Vec2x8::mag of the stored velocity
        speed_out = (m == m) ? m : 0.0f;
        bad = (isfinite(nx) && isfinite(ny)) ? 0u : 1u;
    }
    block_max_count(speed_out, bad, ctl);
}

// Max |v| over all npad lanes (a multiple of 8): a grid of one wave, four
// lanes per step with 16-byte loads, one atomic per block.
__global__ void __launch_bounds__(256) k_vmax(const PartPtrs* __restrict__ pp, uint32_t npad, Ctl* __restrict__ ctl) {
    pdl_wait();
    float m = 0.0f;
    const float* vx = pp->f[VX];
    const float* vy = pp->f[VY];
    for (uint32_t i0 = 4u * (blockIdx.x * blockDim.x + threadIdx.x); i0 < npad; i0 += 4u * gridDim.x * blockDim.x) {
        const float4 x = *reinterpret_cast<const float4*>(vx + i0), y = *reinterpret_cast<const float4*>(vy + i0);
        const float xs[4] = {x.x, x.y, x.z, x.w}, ys[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float mg = sqrtf(xs[q] * xs[q] + ys[q] * ys[q]);
            m = fmaxf(m, (mg == mg) ? mg : 0.0f);
        }
    }
    block_max_count(m, 0u, ctl);
}

__global__ void k_zero_vmax(Ctl* ctl) {
    pdl_wait(); ctl->vmax_bits = 0; ctl->nonfinite = 0; }

// Four consecutive slots per thread: 128-bit loads of the sorted slots and
// 128-bit stores of each field (the gathered reads are one float each).
__global__ void __launch_bounds__(256) k_permute(PartPtrs* __restrict__ pp, const uint32_t* __restrict__ vals,
                                                 uint32_t n, uint32_t npad, uint32_t* __restrict__ status) {
    pdl_wait();
    const uint32_t i0 = 4u * (blockIdx.x * blockDim.x + threadIdx.x);
    if (i0 >= npad) return;  // npad is a multiple of 8
    uint32_t src[4];
    bool ok[4];
    if (i0 + 4u <= n) {
        const uint4 v = *reinterpret_cast<const uint4*>(vals + i0);
        src[0] = v.x; src[1] = v.y; src[2] = v.z; src[3] = v.w;
#pragma unroll
        for (int k = 0; k < 4; ++k) ok[k] = true;
    } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            ok[k] = i0 + uint32_t(k) < n;
            src[k] = ok[k] ? vals[i0 + k] : 0u;
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) ok[k] = ok[k] && APIC_IN_BOUNDS(src[k], npad, status);
#pragma unroll
    for (int f = 0; f < NPF; ++f) {
        const float* a = pp->f[f];
        float4 o;
        o.x = ok[0] ? a[src[0]] : 0.0f;
        o.y = ok[1] ? a[src[1]] : 0.0f;
        o.z = ok[2] ? a[src[2]] : 0.0f;
        o.w = ok[3] ? a[src[3]] : 0.0f;
        *reinterpret_cast<float4*>(pp->alt[f] + i0) = o;
    }
}

__global__ void k_swap_tables(PartPtrs* pp) {
    pdl_wait();
    int f = threadIdx.x;
    if (f < NPF) {
        float* t = pp->f[f];
        pp->f[f] = pp->alt[f];
        pp->alt[f] = t;
    }
}

}  // namespace

// Bit length of the largest P2G bin key (row-major cell index).
static int bin_key_bits(const Scene& s) {
    uint32_t mx = s.cells > 0 ? s.cells - 1 : 0;
    int b = 0;
    while (b < 32 && (mx >> b)) ++b;
    return b;
}

// P2G stage; bin_lo / bin_hi and the base fluid mask must be zero (the
// caller clears them), every accumulator entry is written.
cudaError_t launch_p2g(Scene& s) {
    const bool ref = p2g_reference_order(s);
    cudaError_t e = cudaFuncSetAttribute(k_p2g_gather<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(kGatherSmem));
    if (e != cudaSuccess) return e;
    const uint32_t* svals = s.bin_vals;
    if (s.n > 0) {
        launch(s.use_pdl, k_p2g_bin_keys, div_up(s.n, 1024), 256, 0, s.stream, static_cast<const PartPtrs*>(s.pp), s.n,
               int(s.W), int(s.H), s.dx, s.bin_keys, s.bin_vals, s.lv[0].fluid);
        uint32_t *kres, *vres;
        e = radix_sort_pairs(s.bin_keys, s.bin_vals, s.bin_keys_alt, s.bin_vals_alt, s.sort_hist, s.sort_scan_tmp, s.n,
                             bin_key_bits(s), s.stream, s.use_pdl, &kres, &vres, &s.ctl->status);
        if (e != cudaSuccess) return e;
        launch(s.use_pdl, k_p2g_bounds, div_up(s.n, 256), 256, 0, s.stream, static_cast<const uint32_t*>(kres), s.n,
               s.bin_lo, s.bin_hi, s.cells, &s.ctl->status);
        svals = vres;
    }
    GatherOut o{s.acc_u, s.acc_uw, s.acc_v, s.acc_vw, s.density};
    dim3 grid(div_up(s.W, kGatherTW), div_up(s.H, kGatherTH));
    if (ref)
        launch(s.use_pdl && s.n > 0, k_p2g_gather<true>, grid, kGatherThreads, kGatherSmem, s.stream,
               static_cast<const PartPtrs*>(s.pp), svals, static_cast<const uint32_t*>(s.bin_lo),
               static_cast<const uint32_t*>(s.bin_hi), int(s.W), int(s.H), s.dx, s.ctl, o, s.n, s.npad);
    else
        launch(s.use_pdl && s.n > 0, s.cells > (2u << 20) ? k_p2g_cells<3> : k_p2g_cells<2>, grid, kCellThreads, 0,
               s.stream,
               static_cast<const PartPtrs*>(s.pp), svals, static_cast<const uint32_t*>(s.bin_lo),
               static_cast<const uint32_t*>(s.bin_hi), int(s.W), int(s.H), s.dx, s.ctl, o, s.n, s.npad);
    return cudaGetLastError();
}

cudaError_t launch_g2p(Scene& s) {
    if (s.npad == 0) return cudaSuccess;
    launch(s.use_pdl, k_g2p, div_up(s.npad, 256), 256, 0, s.stream, s.pp, s.npad, int(s.W), int(s.H), s.dx, s.props.border_damping,
                                                      s.ctl, s.u, s.v, s.u_open, s.v_open);
    return cudaGetLastError();
}

// Zero the running maximum, then reduce over the current velocities.
cudaError_t launch_vmax(Scene& s) {
    launch(s.use_pdl, k_zero_vmax, 1, 1, 0, s.stream, s.ctl);
    if (s.npad) {
        const uint32_t g = std::min(div_up(s.npad, 1024), uint32_t(kMaxRedBlocks));
        launch(s.use_pdl, k_vmax, g, 256, 0, s.stream, s.pp, s.npad, s.ctl);
    }
    return cudaGetLastError();
}

// Interleave two SoA particle fields into the reference's Vec2x8 layout
// (per chunk: 8 x lanes then 8 y lanes), for one contiguous copy to the host.
// Thread t writes 16 bytes of the packed output: chunk t / 4, quarter t % 4
// (quarters 0-1: x lanes 0-3, 4-7; quarters 2-3: y lanes).
__global__ void __launch_bounds__(256) k_pack_vec2x8(const PartPtrs* __restrict__ pp, int fx, int fy, uint32_t nchunks,
                                                     float* __restrict__ out) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nchunks * 4u) return;
    const uint32_t c = t >> 2, q = t & 3u;
    const float* src = (q < 2u ? pp->f[fx] : pp->f[fy]) + c * 8u + (q & 1u) * 4u;
    *reinterpret_cast<float4*>(out + size_t(t) * 4u) = *reinterpret_cast<const float4*>(src);
}

cudaError_t launch_pack_vec2x8(Scene& s, int which, float* out) {
    if (s.nchunks == 0) return cudaSuccess;
    k_pack_vec2x8<<<div_up(uint64_t(s.nchunks) * 4, 256), 256, 0, s.stream>>>(s.pp, 2 * which, 2 * which + 1,
                                                                            s.nchunks, out);
    return cudaGetLastError();
}

cudaError_t launch_permute(Scene& s, const uint32_t* sorted_vals) {
    if (s.npad == 0) return cudaSuccess;
    launch(s.use_pdl, k_permute, div_up(s.npad / 4, 256), 256, 0, s.stream, s.pp, sorted_vals, s.n, s.npad,
           &s.ctl->status);
    launch(s.use_pdl, k_swap_tables, 1, 32, 0, s.stream, s.pp);
    return cudaGetLastError();
}

}  // namespace apic
