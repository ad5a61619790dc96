// vcycle_dsm.cu — the middle multigrid levels in distributed shared memory.
//
// The same V-cycle arithmetic as vcycle.cu (smooth_level src/apic.rs:471-535,
// restrict :537-594, prolongate :596-616, solve_coarse_exact :618-704), with
// the levels between the base kernels and the coarse tail held in the shared
// memory of one 16-CTA thread-block cluster.  CTA r owns rows
// [r*R, (r+1)*R) of every such level (R = height / 16): their error and
// residual, and their mask and coefficients plus one halo row on each side.
// A stencil read that falls in another CTA's rows goes to that CTA's shared
// memory (distributed shared memory, a few hundred cycles instead of an L2
// round trip); phases are separated by cluster barriers, whose release /
// acquire order makes every CTA's writes visible to the others.  CTA 0 then
// runs the coarse tail (levels of fewer than 64 rows) exactly as
// k_vcycle_tail does, through global memory.
//
// A phase over a level costs a few hundred cycles of shared-memory latency
// plus one cluster barrier, where the same phase as a kernel (or a phase of
// k_vcycle_mid on L2-resident arrays) costs an L2 round trip per dependent
// load plus a launch.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "apic_device.cuh"
#include "apic_internal.h"
#include "vcycle_common.cuh"

namespace apic {
using namespace vc;
namespace {
namespace cg = cooperative_groups;

constexpr uint32_t kDsmCtas = 16;
constexpr uint32_t kDsmTailRows = 64;
constexpr int kDsmMaxLevels = 6;
constexpr size_t kDsmSmemBudget = 220 * 1024;

// Host-computed layout of one distributed level (byte offsets into the
// dynamic shared memory, identical in every CTA).  Widths are multiples of
// 32, so every row starts on a mask word.
struct DsmLevel {
    int w, h, cells, R;
    int rw_shift, half_shift;  // log2(R*w), log2(w/2), or -1 when not a power of two
    const uint32_t* fluid;
    const float *diag, *inv, *px, *py;  // global, padded layout
    float *res, *err;                   // global, padded layout
    uint32_t o_fl, o_diag, o_inv, o_px, o_py, o_res, o_err;
};

struct DsmParams {
    int n;  // distributed levels; lv[0] is V-cycle level `first`
    int first;
    DsmLevel lv[kDsmMaxLevels];
    // the first tail level (coarse level of lv[n-1]), in global memory
    int tw, tcells;
    const uint32_t* tfluid;
    float* tres;
    const float* terr;
};

// This CTA's view of a distributed level.  Coefficients and mask bits are
// indexed by li = (y - y0 + 1) * w + x (rows y0-1 .. y0+R; rows outside the
// grid hold zero bits), error and residual by (y - y0) * w + x.  A raw index
// r = y * w + x moves to li by r - lo + w.
struct View {
    int w, h, cells, R, y0, lo, rw;
    int rw_shift, half_shift;
    const uint32_t* flw;
    const float *diag, *inv, *px, *py;
    float *res, *err;
};

__device__ __forceinline__ View view_of(const DsmLevel& L, uint8_t* sm, uint32_t rank) {
    View v;
    v.w = L.w;
    v.h = L.h;
    v.cells = L.cells;
    v.R = L.R;
    v.y0 = int(rank) * L.R;
    v.lo = v.y0 * L.w;
    v.rw = L.R * L.w;
    v.rw_shift = L.rw_shift;
    v.half_shift = L.half_shift;
    v.flw = reinterpret_cast<const uint32_t*>(sm + L.o_fl);
    v.diag = reinterpret_cast<const float*>(sm + L.o_diag);
    v.inv = reinterpret_cast<const float*>(sm + L.o_inv);
    v.px = reinterpret_cast<const float*>(sm + L.o_px);
    v.py = reinterpret_cast<const float*>(sm + L.o_py);
    v.res = reinterpret_cast<float*>(sm + L.o_res);
    v.err = reinterpret_cast<float*>(sm + L.o_err);
    return v;
}

__device__ __forceinline__ bool flb(const View& v, int li) { return (v.flw[li >> 5] >> (li & 31)) & 1u; }

// Error at raw index r of this level: own rows from this CTA's shared
// memory, other rows from the owning CTA's (rank r / (R*w)); 0 outside the
// grid (the callers drop non-fluid values).
__device__ __forceinline__ float err_raw(const View& v, const cg::cluster_group& cl, int r) {
    const int rel = r - v.lo;
    if (rel >= 0 && rel < v.rw) return v.err[rel];
    if (r < 0 || r >= v.cells) return 0.0f;
    const int rank = v.rw_shift >= 0 ? (r >> v.rw_shift) : (r / v.rw);
    const float* remote = cl.map_shared_rank(v.err, rank);
    return remote[r - rank * v.rw];
}

// (x, y) of the i-th cell of an area `half` cells wide.
__device__ __forceinline__ void split(int i, int half, int shift, int& row, int& col) {
    if (shift >= 0) {
        row = i >> shift;
        col = i & (half - 1);
    } else {
        row = i / half;
        col = i - row * half;
    }
}

// One SOR update of own cell (x, y): sor_cell_all's arithmetic and neighbour
// order (raw+1, raw+w, raw-1, raw-w, where raw +- 1 wraps between rows as
// the reference's flat index does).  nb(r, xn, yn) gives a neighbour's error.
template <class NB>
__device__ __forceinline__ float sor_dsm(const View& v, int x, int y, float old, bool neighbours, NB nb) {
    const int li = (y - v.y0 + 1) * v.w + x;
    const int raw = y * v.w + x;
    const int W = v.w;
    const float inv = v.inv[li];
    float sum = v.res[li - W];
    if (neighbours) {
        const bool fr = flb(v, li + 1), fu = flb(v, li + W), fl = flb(v, li - 1), fd = flb(v, li - W);
        const float pxc = v.px[li], pyc = v.py[li], pxl = v.px[li - 1], pyd = v.py[li - W];
        const bool xr = x + 1 < W, xl = x > 0;
        const float er = nb(raw + 1, xr ? x + 1 : 0, xr ? y : y + 1);
        const float eu = nb(raw + W, x, y + 1);
        const float el = nb(raw - 1, xl ? x - 1 : W - 1, xl ? y : y - 1);
        const float ed = nb(raw - W, x, y - 1);
        float t = __fmaf_rn(-pxc, er, sum);
        sum = fr ? t : sum;
        t = __fmaf_rn(-pyc, eu, sum);
        sum = fu ? t : sum;
        t = __fmaf_rn(-pxl, el, sum);
        sum = fl ? t : sum;
        t = __fmaf_rn(-pyd, ed, sum);
        sum = fd ? t : sum;
    }
    const float gs = sum * inv;
    const float nv = old + (kOmega * (gs - old));
    return inv == 0.0f ? old : nv;
}

// One colour sweep over own cells (init: the level's error was zero-filled).
__device__ __forceinline__ void dsm_sweep(const View& v, const cg::cluster_group& cl, int color, bool init) {
    const int half = v.w >> 1;
    const int n = v.R * half;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        int row, k;
        split(i, half, v.half_shift, row, k);
        const int y = v.y0 + row;
        const int x = 2 * k + ((y + color) & 1);
        const int o = row * v.w + x;
        if (!flb(v, o + v.w)) continue;  // only fluid cells store
        const float old = init ? 0.0f : v.err[o];
        v.err[o] = sor_dsm(v, x, y, old, !(init && color == 0), [&](int r, int, int) { return err_raw(v, cl, r); });
    }
}

// Restriction of fine view f into the coarse cells of this CTA's coarse rows
// (their children are this CTA's fine rows): restrict_cell_all's arithmetic.
// Coarse view c (with_red: also its first red sweep) or, when c is null, the
// first tail level's residual in CTA 0's shared memory (tail_res, padded
// layout, mapped into this CTA's address space).
__device__ __forceinline__ void dsm_restrict(const View& f, const cg::cluster_group& cl, const View* c,
                                             const DsmParams& p, float* tail_res, uint32_t rank, bool with_red) {
    const int wc = f.w >> 1;
    const int rc = f.R >> 1;
    const int yc0 = int(rank) * rc;
    const int n = rc * wc;
    const int W = f.w;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        int row, cx;
        split(i, wc, f.half_shift, row, cx);
        const int cy = yc0 + row;
        const int craw = cy * wc + cx;
        // only fluid coarse cells store
        if (c ? !flb(*c, craw - c->lo + wc) : !bit_at(p.tfluid, uint32_t(craw))) continue;
        float sum = 0.0f;
#pragma unroll
        for (int dy = 0; dy < 2; ++dy)
#pragma unroll
            for (int dx = 0; dx < 2; ++dx) {
                const int rf = (cy * 2 + dy) * W + (cx * 2 + dx);
                const int li = rf - f.lo + W;
                const bool f0 = flb(f, li);
                const bool fr = flb(f, li + 1), fu = flb(f, li + W), fl = flb(f, li - 1), fd = flb(f, li - W);
                const float b = f.res[li - W];
                float ax = f.diag[li] * f.err[li - W];
                float t = ax + f.px[li] * err_raw(f, cl, rf + 1);
                ax = fr ? t : ax;
                t = ax + f.py[li] * err_raw(f, cl, rf + W);
                ax = fu ? t : ax;
                t = ax + f.px[li - 1] * err_raw(f, cl, rf - 1);
                ax = fl ? t : ax;
                t = ax + f.py[li - W] * err_raw(f, cl, rf - W);
                ax = fd ? t : ax;
                t = sum + (b - ax);
                sum = f0 ? t : sum;
            }
        if (c) {
            const int co = craw - c->lo;
            c->res[co] = sum;
            if (with_red && ((cx + cy) & 1) == 0) {
                const float inv = c->inv[co + wc];
                c->err[co] = inv != 0.0f ? 0.0f + (kOmega * (sum * inv - 0.0f)) : 0.0f;
            }
        } else {
            tail_res[craw + wc] = sum;  // CTA 0's shared memory
        }
    }
}

// Prolongation from the coarse level into own fine cells of one colour,
// fused with that colour's post-sweep (ph_prolong's arithmetic).  Coarse
// error from view c, or (c null) from the first tail level's error in CTA 0's
// shared memory (tail_err, padded layout).
__device__ __forceinline__ void dsm_prolong(const View& f, const cg::cluster_group& cl, const View* c,
                                            const float* tail_err, int color) {
    const int wc = f.w >> 1;
    // coarse error under fine cell (x, y); outside the grid (a neighbour
    // whose value a select drops) reads 0
    auto coarse_e = [&](int x, int y) -> float {
        if (y < 0 || y >= f.h) return 0.0f;
        const int craw = (y >> 1) * wc + (x >> 1);
        return c ? err_raw(*c, cl, craw) : tail_err[craw + wc];
    };
    const int half = f.w >> 1;
    const int n = f.R * half;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        int row, k;
        split(i, half, f.half_shift, row, k);
        const int y = f.y0 + row;
        const int x = 2 * k + ((y + color) & 1);
        const int o = row * f.w + x;
        if (!flb(f, o + f.w)) continue;  // only fluid cells store
        const float old = prolonged(f.err[o], coarse_e(x, y), 0u);
        float z;
        if (color == 1)
            z = sor_dsm(f, x, y, old, true, [&](int r, int xn, int yn) {
                return prolonged(err_raw(f, cl, r), coarse_e(xn, yn), 0u);
            });
        else
            z = sor_dsm(f, x, y, old, true, [&](int r, int, int) { return err_raw(f, cl, r); });
        f.err[o] = z;
    }
}

// Start copying this CTA's rows (plus halo) of every distributed level's mask
// and coefficients into shared memory (they do not change during a solve).
__device__ __forceinline__ void dsm_load_coeffs(const DsmParams& p, uint8_t* sm, uint32_t rank) {
    for (int k = 0; k < p.n; ++k) {
        const DsmLevel& L = p.lv[k];
        const View v = view_of(L, sm, rank);
        const int base = v.lo - L.w;  // raw index of local index 0
        const int nh = (L.R + 2) * L.w;
        // mask words of rows y0-1 .. y0+R (zero outside the grid)
        uint32_t* flw = reinterpret_cast<uint32_t*>(sm + L.o_fl);
        const int words = L.cells >> 5;
        for (int j = threadIdx.x; j < (nh >> 5); j += blockDim.x) {
            const int g = (base >> 5) + j;  // base is a multiple of 32 (w is)
            if (g >= 0 && g < words) cp_async4(flw + j, L.fluid + g);
            else flw[j] = 0u;
        }
        // 16-byte copies: base + w = y0 * w is a multiple of 32 floats and
        // the arrays start 256-byte aligned; padded index base + i + w lies
        // in [0, cells + 2w) for rows -1 .. h
        for (int i = 4 * threadIdx.x; i < nh; i += 4 * blockDim.x) {
            const size_t g = size_t(base + i + L.w);
            cp_async16(const_cast<float*>(v.diag) + i, L.diag + g);
            cp_async16(const_cast<float*>(v.inv) + i, L.inv + g);
            cp_async16(const_cast<float*>(v.px) + i, L.px + g);
            cp_async16(const_cast<float*>(v.py) + i, L.py + g);
        }
    }
}

// Start copying the first level's residual and first red sweep (written by
// the kernel before this one).
__device__ __forceinline__ void dsm_load_first(const DsmParams& p, uint8_t* sm, uint32_t rank) {
    const DsmLevel& L = p.lv[0];
    const View v = view_of(L, sm, rank);
    const int no = L.R * L.w;
    for (int i = 4 * threadIdx.x; i < no; i += 4 * blockDim.x) {
        const size_t g = size_t(v.lo + i + L.w);
        cp_async16(v.res + i, L.res + g);
        cp_async16(v.err + i, L.err + g);
    }
}

__global__ void __launch_bounds__(kTailThreads, 1) k_vcycle_dsm(DsmParams p, TailParams tp, uint32_t dsm_off,
                                                               uint32_t dsm_bytes, const Ctl* ctl) {
    extern __shared__ __align__(16) uint8_t smem[];
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t rank = cl.block_rank();
    uint8_t* dsm = smem + dsm_off;
    uint32_t* tail_sm = reinterpret_cast<uint32_t*>(smem);
    // the first tail level's residual and error live in CTA 0's shared memory
    float* tail_res = cl.map_shared_rank(reinterpret_cast<float*>(tail_sm) + tp.lv[0].o_res, 0);
    const float* tail_err = cl.map_shared_rank(reinterpret_cast<float*>(tail_sm) + tp.lv[0].o_err, 0);
    // Zero the distributed levels first (error and residual of cells outside
    // the fluid mask are never written): with stale shared memory from
    // earlier kernels in place the V-cycle reached NaN on scenes with fluid in
    // every band (noise masks, 512^2), like the coarse tail did; the read
    // that carried the stale value was not located.
    for (uint32_t i = threadIdx.x; i < dsm_bytes / 4; i += blockDim.x) reinterpret_cast<uint32_t*>(dsm)[i] = 0u;
    __syncthreads();
    // masks and coefficients were written by the multigrid setup, before the
    // solve: their copies start while the previous kernel drains
    if (rank == 0) cta_tail_issue_coeffs(tp, tail_sm);
    dsm_load_coeffs(p, dsm, rank);
    pdl_wait();
    if (ctl->pcg_done) {  // the same value in every CTA: all reach every barrier
        cp_async_wait_all();
        return;
    }
    dsm_load_first(p, dsm, rank);
    cp_async_wait_all();
    __syncthreads();
    cl.sync();

    // views are rebuilt from the kernel parameters where needed (an array
    // of them would live in local memory)
    const int n = p.n;
    for (int k = 0; k < n; ++k) {
        const View f = view_of(p.lv[k], dsm, rank);
        dsm_sweep(f, cl, 1, true);  // black sweep; red came with the residual
        cl.sync();
        if (k + 1 < n) {
            const View c = view_of(p.lv[k + 1], dsm, rank);
            dsm_restrict(f, cl, &c, p, tail_res, rank, true);
        } else {
            dsm_restrict(f, cl, nullptr, p, tail_res, rank, false);
        }
        cl.sync();
    }
    if (rank == 0) cta_tail(tp, tail_sm, false, false);
    cl.sync();
    for (int k = n - 1; k >= 0; --k) {
        const View f = view_of(p.lv[k], dsm, rank);
        if (k + 1 < n) {
            const View c = view_of(p.lv[k + 1], dsm, rank);
            dsm_prolong(f, cl, &c, tail_err, 1);
            cl.sync();
            dsm_prolong(f, cl, &c, tail_err, 0);
        } else {
            dsm_prolong(f, cl, nullptr, tail_err, 1);
            cl.sync();
            dsm_prolong(f, cl, nullptr, tail_err, 0);
        }
        cl.sync();  // the next (finer) level reads this one's final error
    }
    // the first level's final error, for the global prolongation above it
    const DsmLevel& L0 = p.lv[0];
    const View v0 = view_of(L0, dsm, rank);
    const int no = L0.R * L0.w;
    for (int i = threadIdx.x; i < no; i += blockDim.x)
        if (flb(v0, i + L0.w)) L0.err[size_t(v0.lo + i + L0.w)] = v0.err[i];
}

size_t dsm_level_bytes(const Level& L, uint32_t R) {
    const size_t nh = size_t(R + 2) * L.w, no = size_t(R) * L.w;
    auto up16 = [](size_t b) { return (b + 15) & ~size_t(15); };
    return up16(nh / 8) + 4 * up16(4 * nh) + 2 * up16(4 * no);
}

int log2_exact(uint32_t v) {
    if (v == 0 || (v & (v - 1))) return -1;
    int k = 0;
    while ((1u << k) < v) ++k;
    return k;
}

cudaLaunchConfig_t dsm_config(size_t smem, cudaStream_t st, cudaLaunchAttribute* attr, bool pdl) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kDsmCtas, 1, 1);
    cfg.blockDim = dim3(kTailThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kDsmCtas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 2 : 1;
    return cfg;
}

}  // namespace

// Pick the distributed levels: the tail starts at the first level with fewer
// than kDsmTailRows rows (one CTA runs a level of 32 x 32 cells with
// __syncthreads between phases faster than the cluster does with cluster
// barriers); going up from there, levels join while their height divides by
// 16 into an even band height, their width is a multiple of 32 and everything
// fits in 220 KB per CTA.
void plan_vcycle_dsm(Scene& s) {
    s.dsm_first = s.dsm_tail = s.nlevels;
    s.dsm_smem = 0;
    s.dsm_off = 0;
    if (s.nlevels < 3) return;
    int d = 1;
    while (d < s.nlevels && s.lv[d].h >= kDsmTailRows) ++d;
    if (d >= s.nlevels || d < 2) return;
    uint32_t tail_words = 0;
    make_tail_params(s, d, &tail_words);
    const size_t off = (size_t(tail_words) * 4 + 15) & ~size_t(15);
    size_t bytes = off;
    int m = d;
    for (int l = d - 1; l >= 1 && d - l <= kDsmMaxLevels; --l) {
        const Level& L = s.lv[l];
        if (L.h % kDsmCtas != 0 || (L.w % 32u) || ((L.h / kDsmCtas) & 1u)) break;
        const size_t b = bytes + dsm_level_bytes(L, L.h / kDsmCtas);
        if (b > kDsmSmemBudget) break;
        bytes = b;
        m = l;
    }
    if (m == d) return;
    cudaFuncSetAttribute(k_vcycle_dsm, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kDsmSmemBudget));
    cudaFuncSetAttribute(k_vcycle_dsm, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaLaunchAttribute attr[2];
    cudaLaunchConfig_t cfg = dsm_config(bytes, nullptr, attr, false);
    int clusters = 0;
    const bool ok = cudaOccupancyMaxActiveClusters(&clusters, k_vcycle_dsm, &cfg) == cudaSuccess && clusters > 0;
    cudaGetLastError();
    if (!ok) return;
    s.dsm_first = m;
    s.dsm_tail = d;
    s.dsm_smem = bytes;
    s.dsm_off = uint32_t(off);
}

// Levels dsm_first .. dsm_tail-1 and the tail in one cluster launch.  On
// entry dsm_first's residual and first red sweep are in global memory
// (k_restrict_red); on exit its final error is.
void launch_vcycle_dsm(Scene& s, cudaStream_t st) {
    DsmParams p = {};
    p.first = s.dsm_first;
    p.n = s.dsm_tail - s.dsm_first;
    uint32_t tail_words = 0;
    TailParams tp = make_tail_params(s, s.dsm_tail, &tail_words);
    size_t o = 0;  // level offsets are relative to the distributed region
    auto take = [&](size_t bytes) {
        const uint32_t at = uint32_t(o);
        o += (bytes + 15) & ~size_t(15);
        return at;
    };
    for (int k = 0; k < p.n; ++k) {
        const Level& L = s.lv[s.dsm_first + k];
        DsmLevel& d = p.lv[k];
        d.w = int(L.w);
        d.h = int(L.h);
        d.cells = int(L.cells);
        d.R = int(L.h / kDsmCtas);
        d.rw_shift = log2_exact(uint32_t(d.R) * L.w);
        d.half_shift = log2_exact(L.w / 2);
        d.fluid = L.fluid;
        d.diag = L.diag;
        d.inv = L.inv_diag;
        d.px = L.px;
        d.py = L.py;
        d.res = L.res;
        d.err = L.err;
        const size_t nh = size_t(d.R + 2) * L.w, no = size_t(d.R) * L.w;
        d.o_fl = take(nh / 8);
        d.o_diag = take(4 * nh);
        d.o_inv = take(4 * nh);
        d.o_px = take(4 * nh);
        d.o_py = take(4 * nh);
        d.o_res = take(4 * no);
        d.o_err = take(4 * no);
    }
    const Level& T = s.lv[s.dsm_tail];
    p.tw = int(T.w);
    p.tcells = int(T.cells);
    p.tfluid = T.fluid;
    p.tres = T.res;
    p.terr = T.err;
    cudaLaunchAttribute attr[2];
    cudaLaunchConfig_t cfg = dsm_config(s.dsm_smem, st, attr, s.use_pdl);
    cudaLaunchKernelEx(&cfg, k_vcycle_dsm, p, tp, s.dsm_off, uint32_t(s.dsm_smem - s.dsm_off),
                       static_cast<const Ctl*>(s.ctl));
}

}  // namespace apic
