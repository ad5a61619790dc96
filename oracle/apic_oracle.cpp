// apic_oracle.cpp — CPU oracle for the APIC/FLIP step (TEST INFRASTRUCTURE).
//
// A C++ restatement of fireblade2534/APIC-Fluid-Simulation `src/apic.rs`,
// function by function, used only as the correctness checker by tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg.  The product
// library never links or calls it.
//
// PARITY UNPINNED: the reference has no tests, fixtures or golden vectors, and
// its Rust toolchain (cargo/rustc) and crates (rdst, wide, ultraviolet, rayon)
// are absent, so this restatement could not be checked against outputs of the
// reference itself.  Where the reference's result depends on third-party
// behaviour that is not vendored, this file fixes one definition and says so:
//   * rdst 0.20.14 `radix_sort_unstable` tie order -> stable (ties by val);
//   * wide 0.7.33 `fast_max`/`fast_min` -> x86 maxps/minps operand rule
//     (a > b ? a : b), `fast_trunc_int` -> cvttps2dq (out of range/NaN ->
//     INT32_MIN), `reduce_add` -> the SSE2 pairing ((l0+l2)+(l1+l3)) +
//     ((l4+l6)+(l5+l7)) (no AVX target feature in Cargo.toml);
//   * ultraviolet 0.10.0 `Vec2x8::mag` -> sqrt(x*x + y*y), `Vec2x8 / f32x8`
//     -> per-component IEEE division;
//   * rayon 1.12.0 reductions -> serial order of the chunk partials.
// Serial mode (threads <= 1) follows the reference's single-thread order
// (P2G chunk by chunk with its in-chunk lane merging, serial list builds).
// OpenMP mode (threads > 1) keeps the reference's parallel/serial split and is
// the timed "C++ restatement of reference CPU step" baseline.
//
// Built with -ffp-contract=off and without -ffast-math; std::fma is used
// exactly where the reference calls mul_add.

#include "apic_oracle.h"

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- helpers --

// expand_bits / morton_code, src/apic.rs:185-203.
inline uint32_t expand_bits(uint32_t v) {
    v &= 0x0000FFFFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}
inline uint32_t morton(uint32_t x, uint32_t y) { return expand_bits(x) | (expand_bits(y) << 1); }

// Apic::random_simd for one lane, src/apic.rs:946-975.
inline float random_lane(uint32_t slot, uint32_t seed) {
    uint32_t m = slot ^ seed;
    m ^= m >> 16;
    m *= 0x7feb352du;
    m ^= m >> 15;
    m *= 0x846ca68bu;
    m ^= m >> 16;
    uint32_t bits = (m & 0x007FFFFFu) | 0x3F800000u;
    float f;
    std::memcpy(&f, &bits, 4);
    return f - 1.5f;
}

// wide::f32x8::fast_max / fast_min on x86 (maxps/minps: second operand on NaN).
template <class T> inline T fmax_x86(T a, T b) { return a > b ? a : b; }
template <class T> inline T fmin_x86(T a, T b) { return a < b ? a : b; }
// wide::f32x8::fast_trunc_int on x86 (cvttps2dq: out of range or NaN -> INT_MIN).
template <class T> inline int32_t trunc_x86(T x) {
    if (!(x >= T(-2147483648.0) && x < T(2147483648.0))) return INT32_MIN;
    return static_cast<int32_t>(x);
}
// i32x8 min-then-max clamp as written in the reference.
inline int32_t clampi(int32_t v, int32_t hi, int32_t lo) { return std::max(std::min(v, hi), lo); }
// Rust f32::clamp.
template <class T> inline T rclamp(T x, T lo, T hi) {
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}

// temporal_kernel_w_t, src/apic.rs:31-46.
template <class T> inline T temporal_w(T tau) {
    T ts = tau - T(0.5);
    T tsq = ts * ts;
    T inner = fmax_x86(T(1) - tsq, T(0));
    T w = inner * inner * inner;
    T wt = w * T(2.1875);
    return fmax_x86(wt, T(1e-5));
}

// dot_product, src/apic.rs:11-29: 8 strided lane sums, SSE2 reduce_add order,
// then the remainder serially.
template <class T> T dot_product(const T* a, const T* b, size_t n) {
    T lane[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    size_t chunks = n / 8;
    for (size_t c = 0; c < chunks; ++c)
        for (int l = 0; l < 8; ++l) lane[l] += a[c * 8 + l] * b[c * 8 + l];
    T result = ((lane[0] + lane[2]) + (lane[1] + lane[3])) + ((lane[4] + lane[6]) + (lane[5] + lane[7]));
    for (size_t i = chunks * 8; i < n; ++i) result += a[i] * b[i];
    return result;
}

inline size_t round8(size_t x) { return (x + 7) / 8 * 8; }

template <class T> inline void atomic_add(T* p, T v, bool par) {
    if (!par) { *p += v; return; }
    std::atomic_ref<T> a(*p);
    T cur = a.load(std::memory_order_relaxed);
    while (!a.compare_exchange_weak(cur, cur + v, std::memory_order_relaxed)) {}
}
inline void atomic_or(uint64_t* p, uint64_t v, bool par) {
    if (!par) { *p |= v; return; }
    std::atomic_ref<uint64_t>(*p).fetch_or(v, std::memory_order_relaxed);
}

// ------------------------------------------------------------- MG level ----

// MultiGridLevel, src/apic.rs:402-705.
template <class T> struct Level {
    size_t width = 0, height = 0, cells = 0;
    std::vector<uint64_t> fluid_bits;
    std::vector<uint32_t> fluid, red, black;
    std::vector<T> diag, inv_diag, px, py, residual, error;
    std::vector<T> cg_s, cg_ap, cg_r;

    void init(size_t w, size_t h) {  // MultiGridLevel::new :428-453
        width = w; height = h; cells = w * h;
        fluid_bits.assign((cells + 63) / 64, 0);
        size_t alloc = round8(cells + 2 * w);
        diag.assign(alloc, 0); inv_diag.assign(alloc, 0); px.assign(alloc, 0); py.assign(alloc, 0);
        residual.assign(alloc, 0); error.assign(alloc, 0);
    }
    void alloc_cg() {  // :455-461
        size_t alloc = round8(cells + 2 * width);
        cg_s.assign(alloc, 0); cg_ap.assign(alloc, 0); cg_r.assign(alloc, 0);
    }
    uint64_t is_fluid_index(size_t i) const {  // :463-469
        size_t w = i >> 6;
        if (w >= fluid_bits.size()) return 0;
        return (fluid_bits[w] >> (i & 63)) & 1;
    }

    // smooth_level, :471-535 (red/black Gauss-Seidel-SOR; each colour is Jacobi).
    void smooth_one(const std::vector<uint32_t>& list, T omega, int threads) {
        const size_t w = width;
        auto body = [&](size_t k) {
            size_t c = list[k];
            T inv = inv_diag[c];
            if (inv != T(0)) {
                T sum = residual[c];
                sum = std::fma(-px[c], error[c + 1], sum);
                sum = std::fma(-py[c], error[c + w], sum);
                sum = std::fma(-px[c - 1], error[c - 1], sum);
                sum = std::fma(-py[c - w], error[c - w], sum);
                T gs = sum * inv;
                T old = error[c];
                error[c] = old + (omega * (gs - old));
            }
        };
        bool par = threads > 1 && red.size() > 4096;
        if (par) {
#pragma omp parallel for num_threads(threads) schedule(static, 4096)
            for (size_t k = 0; k < list.size(); ++k) body(k);
        } else {
            for (size_t k = 0; k < list.size(); ++k) body(k);
        }
    }
    void smooth(bool reverse, T omega, int threads) {
        // `use_parallel` is decided from red_indices.len() for both colours (:514).
        if (reverse) { smooth_one(black, omega, threads); smooth_one(red, omega, threads); }
        else { smooth_one(red, omega, threads); smooth_one(black, omega, threads); }
    }

    // restrict, :537-594.
    void restrict_to(Level& coarse, int threads) const {
        size_t cs = coarse.width, ce = cs + coarse.cells;
        std::fill(coarse.error.begin() + cs, coarse.error.begin() + ce, T(0));
        auto body = [&](size_t k) {
            size_t ci = coarse.fluid[k];
            size_t raw_c = ci - coarse.width;
            size_t cx = raw_c % coarse.width, cy = raw_c / coarse.width;
            T sum = 0;
            for (size_t dy = 0; dy < 2; ++dy)
                for (size_t dx = 0; dx < 2; ++dx) {
                    size_t fx = cx * 2 + dx, fy = cy * 2 + dy;
                    size_t raw_f = fy * width + fx, pf = raw_f + width;
                    if (is_fluid_index(raw_f) == 1) {
                        T b = residual[pf];
                        T ax = diag[pf] * error[pf];
                        ax += px[pf] * error[pf + 1];
                        ax += py[pf] * error[pf + width];
                        ax += px[pf - 1] * error[pf - 1];
                        ax += py[pf - width] * error[pf - width];
                        sum += b - ax;
                    }
                }
            coarse.residual[ci] = sum;
        };
        if (threads > 1 && coarse.fluid.size() > 4096) {
#pragma omp parallel for num_threads(threads) schedule(static, 4096)
            for (size_t k = 0; k < coarse.fluid.size(); ++k) body(k);
        } else {
            for (size_t k = 0; k < coarse.fluid.size(); ++k) body(k);
        }
    }

    // prolongate, :596-616 (iterates this level's fluid list, padded on the base level).
    void prolongate_from(const Level& coarse, int threads) {
        auto body = [&](size_t k) {
            size_t fi = fluid[k];
            size_t raw_f = fi - width;
            size_t cx = (raw_f % width) / 2, cy = (raw_f / width) / 2;
            size_t rc = cy * coarse.width + cx + coarse.width;
            error[fi] += coarse.error[rc];
        };
        if (threads > 1 && fluid.size() > 4096) {
            // Duplicated trailing entries of a padded list must be applied by one
            // thread, as they are in the reference's 4096-element chunks.
#pragma omp parallel for num_threads(threads) schedule(static, 4096)
            for (size_t k = 0; k < fluid.size(); ++k) body(k);
        } else {
            for (size_t k = 0; k < fluid.size(); ++k) body(k);
        }
    }

    // solve_coarse_exact, :618-704 (serial CG).
    void solve_coarse_exact() {
        size_t start = width, end = start + cells;
        std::fill(error.begin() + start, error.begin() + end, T(0));
        std::copy(residual.begin() + start, residual.begin() + end, cg_r.begin() + start);
        std::copy(residual.begin() + start, residual.begin() + end, cg_s.begin() + start);
        T gamma = 0;
        for (uint32_t i : fluid) gamma += cg_r[i] * cg_r[i];
        if (gamma < T(1e-12)) return;
        size_t max_it = std::min<size_t>(fluid.size(), 100);
        size_t w = width;
        for (size_t it = 0; it < max_it; ++it) {
            T delta = 0;
            for (uint32_t i : fluid) {
                T v = diag[i] * cg_s[i];
                v = std::fma(px[i], cg_s[i + 1], v);
                v = std::fma(px[i - 1], cg_s[i - 1], v);
                v = std::fma(py[i], cg_s[i + w], v);
                v = std::fma(py[i - w], cg_s[i - w], v);
                cg_ap[i] = v;
                delta += cg_s[i] * v;
            }
            if (std::fabs(delta) < T(1e-5)) break;
            T alpha = gamma / delta;
            T max_err = 0;
            for (uint32_t i : fluid) {
                error[i] += alpha * cg_s[i];
                cg_r[i] -= alpha * cg_ap[i];
                max_err = std::fmax(max_err, std::fabs(cg_r[i]));
            }
            if (max_err < T(1e-6)) break;
            T ng = 0;
            for (uint32_t i : fluid) ng += cg_r[i] * cg_r[i];
            T beta = ng / gamma;
            gamma = ng;
            for (uint32_t i : fluid) cg_s[i] = cg_r[i] + (beta * cg_s[i]);
        }
    }
};

// --------------------------------------------------------------- the sim ---

struct SimBase {
    virtual ~SimBase() {}
};

template <class T> struct Sim : SimBase {
    // WorldProperties
    T gravity = 0, border_damping = 0, cfl = 0, solve_error = 0;
    uint32_t width = 0, height = 0, cells = 0;
    T cell_size = 0;
    uint32_t num_chunks = 0, num_particles = 0;

    std::vector<T> ext_u, ext_v, post_u, post_v;
    std::vector<T> smoothed, old_density, pressure;
    std::vector<uint64_t> obstacle;
    std::vector<uint8_t> valid_u, valid_v, next_valid_u, next_valid_v;
    std::vector<T> mac_u, mac_v, old_u, old_v;
    std::vector<T> acc_u_vel, acc_u_w, acc_v_vel, acc_v_w;  // mac_{u,v}_and_weight
    std::vector<T> density;
    std::vector<uint64_t> u_open, v_open;  // mac_{u,v}_blocked (bit set = open face)
    std::vector<T> search, ap;

    // particles, SoA over num_chunks*8 lanes (AoSoA-8 lane = index % 8)
    enum { PX, PY, VX, VY, CUX, CUY, CVX, CVY, TR, NPF };
    std::vector<T> part[NPF], part_sort[NPF];
    std::vector<uint32_t> sort_key, sort_val;

    uint32_t fluid_cells = 0;
    Level<T> base;
    std::vector<Level<T>> levels;
    uint32_t timestamp = 0;
    T prev_dt = 0;
    int threads = 1;
    int solver_mode = APIC_SOLVER_REFERENCE;
    T rel_tol = T(1e-6);
    uint32_t max_iter = 500;
    bool world_ready = false;
    apic_step_stats stats{};
    std::vector<double> p64;   // refined FP64 pressure of the mixed mode (padded layout)
    bool p64_valid = false;
    // The mixed mode starts each solve from the previous solve's FP64
    // pressure (the GPU library's APIC_OPT_WARM_START); empty p64: from zero.
    bool warm_start = true;

    bool par() const { return threads > 1; }
    size_t npad() const { return size_t(num_chunks) * 8; }
    size_t u_faces() const { return size_t(cells) + height; }
    size_t v_faces() const { return size_t(cells) + width; }

    // ---- construction, Apic::new :779-916
    void construct(uint32_t w, uint32_t h, float cs, const apic_world_props& p) {
        base.init(w, h);
        gravity = p.gravity; border_damping = p.border_damping; cfl = p.cfl; solve_error = p.solve_error;
        width = w; height = h; cell_size = cs; cells = w * h;
        pressure.assign(round8(cells), 0);
        valid_u.assign(u_faces(), 0); valid_v.assign(v_faces(), 0);
        obstacle.assign((cells + 63) / 64, 0);
        old_u.assign(u_faces(), 0); old_v.assign(v_faces(), 0);
        next_valid_u.assign(u_faces(), 0); next_valid_v.assign(v_faces(), 0);
        mac_u.assign(u_faces(), 0); mac_v.assign(v_faces(), 0);
        acc_u_vel.assign(u_faces(), 0); acc_u_w.assign(u_faces(), 0);
        acc_v_vel.assign(v_faces(), 0); acc_v_w.assign(v_faces(), 0);
        density.assign(round8(cells), 0);
        u_open.assign((u_faces() + 63) / 64, 0); v_open.assign((v_faces() + 63) / 64, 0);
        smoothed.assign(round8(cells), 0); old_density.assign(round8(cells), 0);
        search.assign(round8(cells + 2 * size_t(w)), 0); ap.assign(round8(cells + 2 * size_t(w)), 0);
        prev_dt = T(1.0) / T(60.0);
        ext_u.assign(u_faces(), 0); ext_v.assign(v_faces(), 0);
        post_u.assign(u_faces(), 0); post_v.assign(v_faces(), 0);

        std::vector<T> ix, iy;
        for (uint32_t y = 0; y < h; ++y)
            for (uint32_t x = 0; x < w; ++x) {
                if (x == 0 || x == w - 1 || y == 0 || y == h - 1) {
                    uint32_t idx = y * w + x;
                    obstacle[idx / 64] |= 1ull << (idx % 64);
                } else if (x > 4 && x < w - 4 && y > 4 && y < h / 2) {
                    for (int py = 0; py < 3; ++py)
                        for (int px = 0; px < 3; ++px) {
                            ix.push_back((T(x) + (T(px) + T(0.5)) / T(3.0)) * cell_size);
                            iy.push_back((T(y) + (T(py) + T(0.5)) / T(3.0)) * cell_size);
                        }
                }
            }
        load_positions(ix, iy, nullptr, nullptr);
        if (num_particles == 0) { num_chunks = 0; return; }
        build_levels();
        update_world();
    }

    bool build_levels() {  // :900-911
        levels.clear();
        size_t cw = width, ch = height;
        while (cw % 2 == 0 && ch % 2 == 0 && cw > 4 && ch > 4) {
            cw /= 2; ch /= 2;
            levels.emplace_back();
            levels.back().init(cw, ch);
        }
        if (levels.empty()) return false;  // the reference panics here (usize underflow)
        levels.back().alloc_cg();
        return true;
    }

    void load_positions(const std::vector<T>& ix, const std::vector<T>& iy,
                        const std::vector<T>* ivx, const std::vector<T>* ivy) {
        num_particles = uint32_t(ix.size());
        num_chunks = (num_particles + 7) / 8;
        for (int f = 0; f < NPF; ++f) {
            part[f].assign(npad(), 0);
            part_sort[f].assign(npad(), 0);
        }
        sort_key.assign(num_particles, 0);
        sort_val.assign(num_particles, 0);
        for (size_t i = 0; i < ix.size(); ++i) {
            part[PX][i] = ix[i]; part[PY][i] = iy[i];
            if (ivx) { part[VX][i] = (*ivx)[i]; part[VY][i] = (*ivy)[i]; }
        }
        if (num_particles % 8 != 0) {  // :887-898 pad with the last position
            for (size_t l = num_particles; l < npad(); ++l) {
                part[PX][l] = ix.back(); part[PY][l] = iy.back();
            }
        }
    }

    // update_world, :918-944.
    uint64_t is_obstacle(int32_t i, int32_t j) const {  // :994-1003
        if (i < 0 || i >= int32_t(width) || j < 0 || j >= int32_t(height)) return 1;
        uint32_t idx = uint32_t(j * int32_t(width) + i);
        return (obstacle[idx >> 6] >> (idx & 63)) & 1;
    }
    uint64_t is_obstacle_index(size_t idx) const {  // :1006-1012
        if ((idx >> 6) >= obstacle.size()) return 1;
        return (obstacle[idx >> 6] >> (idx & 63)) & 1;
    }
    uint64_t is_fluid(int32_t i, int32_t j) const {  // :1015-1022
        if (i < 0 || i >= int32_t(width) || j < 0 || j >= int32_t(height)) return 0;
        return base.is_fluid_index(size_t(j) * width + size_t(i));
    }
    void update_world() {
        std::fill(u_open.begin(), u_open.end(), 0);
        for (size_t idx = 0; idx < u_faces(); ++idx) {
            int32_t i = int32_t(idx % (width + 1)), j = int32_t(idx / (width + 1));
            if ((is_obstacle(i - 1, j) | is_obstacle(i, j)) == 0) u_open[idx >> 6] |= 1ull << (idx & 63);
        }
        std::fill(v_open.begin(), v_open.end(), 0);
        for (size_t idx = 0; idx < v_faces(); ++idx) {
            int32_t i = int32_t(idx % width), j = int32_t(idx / width);
            if ((is_obstacle(i, j - 1) | is_obstacle(i, j)) == 0) v_open[idx >> 6] |= 1ull << (idx & 63);
        }
        world_ready = true;
    }

    // ---- u/v staggered stencils, get_u_grid / get_v_grid / get_grid_distances :1113-1216
    struct Stencil {
        uint32_t idx[4];   // bl, br, tl, tr
        T w[4];            // bilinear weights
        T dx[4], dy[4];    // node - particle offsets in world units
        T tx, ty;
    };
    uint32_t u_index(int32_t i, int32_t j) const {  // u_index_simd :1030-1034
        uint32_t ci = uint32_t(clampi(i, int32_t(width), 0));
        uint32_t cj = uint32_t(clampi(j, int32_t(height - 1), 0));
        return cj * (width + 1) + ci;
    }
    uint32_t v_index(int32_t i, int32_t j) const {  // v_index_simd :1037-1041
        uint32_t ci = uint32_t(clampi(i, int32_t(width - 1), 0));
        uint32_t cj = uint32_t(clampi(j, int32_t(height), 0));
        return cj * width + ci;
    }
    void distances(T tx, T ty, Stencil& s) const {
        T dx = cell_size;
        T itx = T(1) - tx, ity = T(1) - ty;
        s.dx[0] = -tx * dx; s.dy[0] = -ty * dx;
        s.dx[1] = itx * dx; s.dy[1] = -ty * dx;
        s.dx[2] = -tx * dx; s.dy[2] = ity * dx;
        s.dx[3] = itx * dx; s.dy[3] = ity * dx;
    }
    void weights(T tx, T ty, Stencil& s) const {
        T itx = T(1) - tx, ity = T(1) - ty;
        s.w[0] = itx * ity; s.w[1] = tx * ity; s.w[2] = itx * ty; s.w[3] = tx * ty;
    }
    void u_stencil(T gx, T gy, Stencil& s) const {
        T ugx = gx, ugy = gy - T(0.5);
        T bx = std::floor(ugx), by = std::floor(ugy);
        int32_t ix = trunc_x86(bx), iy = trunc_x86(by);
        s.idx[0] = u_index(ix, iy); s.idx[1] = u_index(ix + 1, iy);
        s.idx[2] = u_index(ix, iy + 1); s.idx[3] = u_index(ix + 1, iy + 1);
        s.tx = ugx - bx; s.ty = ugy - by;
        weights(s.tx, s.ty, s);
        distances(s.tx, s.ty, s);
    }
    void v_stencil(T gx, T gy, Stencil& s) const {
        T vgx = gx - T(0.5), vgy = gy;
        T bx = std::floor(vgx), by = std::floor(vgy);
        s.tx = vgx - bx; s.ty = vgy - by;
        weights(s.tx, s.ty, s);
        int32_t ix = trunc_x86(bx), iy = trunc_x86(by);
        s.idx[0] = v_index(ix, iy); s.idx[1] = v_index(ix + 1, iy);
        s.idx[2] = v_index(ix, iy + 1); s.idx[3] = v_index(ix + 1, iy + 1);
        distances(s.tx, s.ty, s);
    }

    // ---- get_max_particle_velocity, :2412-2427
    T max_particle_velocity() const {
        T lanes[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (size_t c = 0; c < num_chunks; ++c)
            for (int l = 0; l < 8; ++l) {
                size_t i = c * 8 + l;
                T vx = part[VX][i], vy = part[VY][i];
                T mag = std::sqrt(vx * vx + vy * vy);
                lanes[l] = fmax_x86(lanes[l], mag);
            }
        T m = 0;
        for (int l = 0; l < 8; ++l) m = std::fmax(m, lanes[l]);
        return m;
    }

    // ---- update_spatial_lookup, :1043-1111 (stable LSD radix sort in place of rdst)
    void spatial_lookup() {
        T max_x = T(width > 0 ? width - 1 : 0), max_y = T(height > 0 ? height - 1 : 0);
        size_t n = num_particles;
        for (size_t i = 0; i < n; ++i) {
            T gx = part[PX][i] / cell_size, gy = part[PY][i] / cell_size;
            uint32_t cx = uint32_t(trunc_x86(fmin_x86(fmax_x86(gx, T(0)), max_x)));
            uint32_t cy = uint32_t(trunc_x86(fmin_x86(fmax_x86(gy, T(0)), max_y)));
            sort_key[i] = morton(cx, cy);
            sort_val[i] = uint32_t(i);
        }
        radix_sort_pairs();
        for (int f = 0; f < NPF; ++f) {
            std::vector<T>& dst = part_sort[f];
            const std::vector<T>& src = part[f];
            for (size_t i = 0; i < npad(); ++i) dst[i] = i < n ? src[sort_val[i]] : T(0);
            std::swap(part[f], part_sort[f]);
        }
    }
    void radix_sort_pairs() {
        size_t n = sort_key.size();
        std::vector<uint32_t> k2(n), v2(n);
        for (int shift = 0; shift < 32; shift += 8) {
            size_t count[257] = {0};
            bool all_same = true;
            for (size_t i = 0; i < n; ++i) {
                uint32_t d = (sort_key[i] >> shift) & 0xFF;
                count[d + 1]++;
                if (i && d != ((sort_key[0] >> shift) & 0xFF)) all_same = false;
            }
            if (all_same) continue;  // a pass over one digit value leaves the order unchanged
            for (int d = 0; d < 256; ++d) count[d + 1] += count[d];
            for (size_t i = 0; i < n; ++i) {
                uint32_t d = (sort_key[i] >> shift) & 0xFF;
                size_t o = count[d]++;
                k2[o] = sort_key[i];
                v2[o] = sort_val[i];
            }
            sort_key.swap(k2);
            sort_val.swap(v2);
        }
    }

    // ---- transfer_particles_to_grid, :1218-1497
    static void add_to_mac(T* acc_vel, T* acc_w, const uint32_t* idx, const T* val, const T* w,
                           size_t active, bool par) {  // :296-344
        uint32_t processed = 0;
        for (size_t l = 0; l < active; ++l) {
            if (processed & (1u << l)) continue;
            uint32_t index = idx[l];
            T value = val[l], weight = w[l];
            for (size_t o = l + 1; o < active; ++o)
                if (idx[o] == index) { value += val[o]; weight += w[o]; processed |= 1u << o; }
            if (value != T(0) || weight != T(0)) {
                if (!par) { acc_vel[index] = acc_vel[index] + value; acc_w[index] = acc_w[index] + weight; }
                else {
                    // The reference packs (vel, weight) into one 64-bit CAS; two atomics
                    // give the same sums up to order.
                    atomic_add(&acc_vel[index], value, true);
                    atomic_add(&acc_w[index], weight, true);
                }
            }
        }
    }
    static void add_to_vec(T* acc, const uint32_t* idx, const T* w, size_t active, bool par) {  // :347-369
        uint32_t processed = 0;
        for (size_t l = 0; l < active; ++l) {
            if (processed & (1u << l)) continue;
            uint32_t index = idx[l];
            T weight = w[l];
            for (size_t o = l + 1; o < active; ++o)
                if (idx[o] == index) { weight += w[o]; processed |= 1u << o; }
            if (weight == T(0)) continue;  // atomic_add_f32 early return, :273-275
            atomic_add(&acc[index], weight, par);
        }
    }
    static void add_to_fluid(uint64_t* bits, const uint32_t* idx, size_t active, bool par) {  // :372-395
        uint32_t processed = 0;
        for (size_t l = 0; l < active; ++l) {
            if (processed & (1u << l)) continue;
            size_t wi = idx[l] / 64;
            uint64_t mask = 1ull << (idx[l] % 64);
            for (size_t o = l + 1; o < active; ++o)
                if (idx[o] / 64 == wi) { mask |= 1ull << (idx[o] % 64); processed |= 1u << o; }
            atomic_or(&bits[wi], mask, par);
        }
    }

    void p2g_chunk(size_t c) {
        uint32_t fidx[8], ui[4][8], vi[4][8], ci[4][8];
        T ua[4][8], uw[4][8], va[4][8], vw[4][8], cw[4][8];
        const T half = T(0.5), one = T(1);
        for (int l = 0; l < 8; ++l) {
            size_t i = c * 8 + l;
            T px = part[PX][i], py = part[PY][i], vx = part[VX][i], vy = part[VY][i];
            T cux = part[CUX][i], cuy = part[CUY][i], cvx = part[CVX][i], cvy = part[CVY][i];
            T tau = (-part[TR][i]) / prev_dt;
            T wt = temporal_w(tau);
            T gx = px / cell_size, gy = py / cell_size;
            // cell-centred density stencil :1260-1284
            T cgx = gx - half, cgy = gy - half;
            T cbx = std::floor(cgx), cby = std::floor(cgy);
            T ctx = cgx - cbx, cty = cgy - cby;
            cw[0][l] = ((one - ctx) * (one - cty)) * wt;
            cw[1][l] = (ctx * (one - cty)) * wt;
            cw[2][l] = ((one - ctx) * cty) * wt;
            cw[3][l] = (ctx * cty) * wt;
            int32_t mx = int32_t(width) - 1, my = int32_t(height) - 1;
            int32_t tbx = trunc_x86(cbx), tby = trunc_x86(cby);
            int32_t cx0 = clampi(tbx, mx, 0), cx1 = clampi(tbx + 1, mx, 0);
            int32_t cy0 = clampi(tby, my, 0), cy1 = clampi(tby + 1, my, 0);
            int32_t W = int32_t(width);
            ci[0][l] = uint32_t(cy0 * W + cx0); ci[1][l] = uint32_t(cy0 * W + cx1);
            ci[2][l] = uint32_t(cy1 * W + cx0); ci[3][l] = uint32_t(cy1 * W + cx1);
            Stencil su, sv;
            u_stencil(gx, gy, su);
            v_stencil(gx, gy, sv);
            for (int k = 0; k < 4; ++k) {
                T wu = su.w[k] * wt, wv = sv.w[k] * wt;
                ui[k][l] = su.idx[k]; vi[k][l] = sv.idx[k];
                uw[k][l] = wu; vw[k][l] = wv;
                ua[k][l] = (vx + cux * su.dx[k] + cuy * su.dy[k]) * wu;
                va[k][l] = (vy + cvx * sv.dx[k] + cvy * sv.dy[k]) * wv;
            }
            T clx = fmax_x86(fmin_x86(gx, T(width) - T(1.0)), T(0));
            T cly = fmax_x86(fmin_x86(gy, T(height) - T(1.0)), T(0));
            fidx[l] = uint32_t(trunc_x86(cly) * int32_t(width) + trunc_x86(clx));
        }
        size_t active = (c == num_chunks - 1 && num_particles % 8 != 0) ? num_particles % 8 : 8;
        bool p = par();
        add_to_fluid(base.fluid_bits.data(), fidx, active, p);
        for (int k = 0; k < 4; ++k) add_to_mac(acc_u_vel.data(), acc_u_w.data(), ui[k], ua[k], uw[k], active, p);
        for (int k = 0; k < 4; ++k) add_to_mac(acc_v_vel.data(), acc_v_w.data(), vi[k], va[k], vw[k], active, p);
        for (int k = 0; k < 4; ++k) add_to_vec(density.data(), ci[k], cw[k], active, p);
    }

    void p2g() {
        std::fill(base.fluid_bits.begin(), base.fluid_bits.end(), 0);
        base.red.clear(); base.black.clear(); base.fluid.clear();
        std::fill(mac_u.begin(), mac_u.end(), T(0)); std::fill(mac_v.begin(), mac_v.end(), T(0));
        std::fill(acc_u_vel.begin(), acc_u_vel.end(), T(0)); std::fill(acc_u_w.begin(), acc_u_w.end(), T(0));
        std::fill(acc_v_vel.begin(), acc_v_vel.end(), T(0)); std::fill(acc_v_w.begin(), acc_v_w.end(), T(0));
        std::fill(density.begin(), density.end(), T(0));
        std::fill(valid_u.begin(), valid_u.end(), 0); std::fill(valid_v.begin(), valid_v.end(), 0);
        if (par()) {
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
            for (size_t c = 0; c < num_chunks; ++c) p2g_chunk(c);
        } else {
            for (size_t c = 0; c < num_chunks; ++c) p2g_chunk(c);
        }
        // normalise :1428-1459
#pragma omp parallel for num_threads(threads) if (par())
        for (size_t f = 0; f < u_faces(); ++f)
            if (acc_u_w[f] > T(0)) { valid_u[f] = 1; mac_u[f] = acc_u_vel[f] / acc_u_w[f]; }
#pragma omp parallel for num_threads(threads) if (par())
        for (size_t f = 0; f < v_faces(); ++f)
            if (acc_v_w[f] > T(0)) { valid_v[f] = 1; mac_v[f] = acc_v_vel[f] / acc_v_w[f]; }
        // serial fluid / red / black lists :1461-1494
        fluid_cells = 0;
        for (size_t i = 0; i < base.fluid_bits.size(); ++i) {
            base.fluid_bits[i] &= ~obstacle[i];
            uint64_t m = base.fluid_bits[i];
            while (m) {
                size_t raw = i * 64 + size_t(__builtin_ctzll(m));
                uint32_t padded = uint32_t(raw + width);
                base.fluid.push_back(padded);
                ++fluid_cells;
                size_t x = raw % width, y = raw / width;
                ((x + y) % 2 == 0 ? base.red : base.black).push_back(padded);
                m &= m - 1;
            }
        }
        uint32_t rem = fluid_cells % 8;
        if (rem) {
            uint32_t last = base.fluid[fluid_cells - 1];
            for (uint32_t k = 0; k < 8 - rem; ++k) base.fluid.push_back(last);
        }
    }

    // ---- apply_external_forces, :1604-1626
    void external_forces(T dt) {
        T g = gravity * dt;
        for (size_t i = 0; i < mac_u.size(); ++i) mac_u[i] += ext_u[i] * dt;
        for (size_t i = 0; i < mac_v.size(); ++i) mac_v[i] += ext_v[i] * dt;
        for (int32_t y = 0; y <= int32_t(height); ++y)
            for (int32_t x = 0; x < int32_t(width); ++x) {
                size_t f = v_index(x, y);
                if (is_fluid(x, y - 1) == 1 || is_fluid(x, y) == 1) mac_v[f] += g;
            }
    }

    // ---- calculate_theta, :1628-1638
    static T theta(T rho, T rho_center, T target) {
        T threshold = target * T(0.5);
        T diff = rho_center - rho;
        if (std::fabs(diff) <= T(1e-5)) return T(1);
        return rclamp((rho_center - threshold) / diff, T(0.1), T(1.0));
    }

    // ---- build_pressure_system, :1640-1785
    void build_pressure() {
        size_t start = width, end = start + cells, W = width;
        std::fill(base.diag.begin() + start, base.diag.begin() + end, T(0));
        std::fill(base.inv_diag.begin() + start, base.inv_diag.begin() + end, T(0));
        std::fill(base.px.begin() + start, base.px.begin() + end, T(0));
        std::fill(base.py.begin() + start, base.py.begin() + end, T(0));
        smoothed = density;
        old_density = density;
        bool pf = par() && base.fluid.size() > 4096;
        for (int pass = 0; pass < 3; ++pass) {
            std::swap(smoothed, old_density);
            T* sm = smoothed.data();
            const T* od = old_density.data();
#pragma omp parallel for num_threads(threads) if (pf) schedule(static, 4096)
            for (size_t k = 0; k < fluid_cells; ++k) {
                size_t raw = base.fluid[k] - W;
                T sum = od[raw] * T(4.0);
                T weight = T(4.0);
                T fl = T(base.is_fluid_index(raw - 1)), fr = T(base.is_fluid_index(raw + 1));
                T fb = T(base.is_fluid_index(raw - W)), ft = T(base.is_fluid_index(raw + W));
                sum += od[raw - 1] * fl;
                sum += od[raw + 1] * fr;
                sum += od[raw - W] * fb;
                sum += od[raw + W] * ft;
                weight += fl + fr + fb + ft;
                sm[raw] = sum / weight;
            }
        }
        const T target = T(9.0);
        const T noise = target * T(1.15);
        const T corr = T(0.1);
        const T cs = cell_size;
#pragma omp parallel for num_threads(threads) if (pf) schedule(static, 4096)
        for (size_t k = 0; k < fluid_cells; ++k) {
            size_t fi = base.fluid[k];
            size_t raw = fi - W;
            size_t gx = raw % W, gy = raw / W;
            size_t ui = gy * (W + 1) + gx;
            T ul = mac_u[ui], ur = mac_u[ui + 1], vb = mac_v[raw], vt = mac_v[raw + W];
            uint64_t nol = 1 - is_obstacle_index(raw - 1), nor = 1 - is_obstacle_index(raw + 1);
            uint64_t nob = 1 - is_obstacle_index(raw - W), not_ = 1 - is_obstacle_index(raw + W);
            ul *= T(nol); ur *= T(nor); vb *= T(nob); vt *= T(not_);
            T div = (ur - ul) + (vt - vb);
            T rc = smoothed[raw];
            T excess = std::fmin(std::fmax(rc - noise, T(0)), target);
            uint64_t fl = base.is_fluid_index(raw - 1), fr = base.is_fluid_index(raw + 1);
            uint64_t fb = base.is_fluid_index(raw - W), ft = base.is_fluid_index(raw + W);
            T diag = 0, px = 0, py = 0;
            if (nol == 1) { if (fl == 1) diag += T(1); else diag += T(1) / theta(smoothed[raw - 1], rc, target); }
            if (nor == 1) { if (fr == 1) { diag += T(1); px = T(-1); } else diag += T(1) / theta(smoothed[raw + 1], rc, target); }
            if (nob == 1) { if (fb == 1) diag += T(1); else diag += T(1) / theta(smoothed[raw - W], rc, target); }
            if (not_ == 1) { if (ft == 1) { diag += T(1); py = T(-1); } else diag += T(1) / theta(smoothed[raw + W], rc, target); }
            base.residual[fi] = -div * cs + excess * corr * cs * cs;
            base.px[fi] = px;
            base.py[fi] = py;
            base.diag[fi] = diag;
            base.inv_diag[fi] = diag > T(1e-6) ? T(1) / diag : T(0);
        }
    }

    // ---- update_multilevel_grid, :1499-1602 (serial)
    void update_multilevel() {
        uint32_t w = width;
        for (size_t li = 0; li < levels.size(); ++li) {
            const Level<T>& fine = li == 0 ? base : levels[li - 1];
            Level<T>& coarse = levels[li];
            coarse.fluid.clear(); coarse.red.clear(); coarse.black.clear();
            std::fill(coarse.fluid_bits.begin(), coarse.fluid_bits.end(), 0);
            size_t cs = coarse.width, ce = cs + coarse.cells;
            std::fill(coarse.diag.begin() + cs, coarse.diag.begin() + ce, T(0));
            std::fill(coarse.inv_diag.begin() + cs, coarse.inv_diag.begin() + ce, T(0));
            std::fill(coarse.px.begin() + cs, coarse.px.begin() + ce, T(0));
            std::fill(coarse.py.begin() + cs, coarse.py.begin() + ce, T(0));
            uint32_t nw = uint32_t(coarse.width);
            for (uint32_t ci : fine.fluid) {
                uint32_t raw = ci - w;
                uint32_t nx = (raw % w) / 2, ny = (raw / w) / 2;
                uint32_t ni = ny * nw + nx;
                coarse.fluid_bits[ni / 64] |= 1ull << (ni % 64);
            }
            for (size_t i = 0; i < coarse.fluid_bits.size(); ++i) {
                uint64_t m = coarse.fluid_bits[i];
                while (m) {
                    uint32_t raw = uint32_t(i * 64 + size_t(__builtin_ctzll(m)));
                    uint32_t padded = raw + nw;
                    coarse.fluid.push_back(padded);
                    uint32_t x = raw % nw, y = raw / nw;
                    ((x + y) % 2 == 0 ? coarse.red : coarse.black).push_back(padded);
                    m &= m - 1;
                }
            }
            for (uint32_t ci : coarse.fluid) {
                size_t cx = (ci - coarse.width) % coarse.width, cy = (ci - coarse.width) / coarse.width;
                T diag = 0, px = 0, py = 0;
                for (size_t dy = 0; dy < 2; ++dy)
                    for (size_t dx = 0; dx < 2; ++dx) {
                        size_t fx = cx * 2 + dx, fy = cy * 2 + dy;
                        if (fx >= fine.width || fy >= fine.height) continue;
                        size_t fr = fy * fine.width + fx, fp = fr + fine.width;
                        if (fine.is_fluid_index(fr) == 1) {
                            diag += fine.diag[fp];
                            if (dx == 0) diag += T(2.0) * fine.px[fp];
                            if (dy == 0) diag += T(2.0) * fine.py[fp];
                            if (dx == 1) px += fine.px[fp];
                            if (dy == 1) py += fine.py[fp];
                        }
                    }
                T fd = diag * T(0.5);
                coarse.diag[ci] = fd;
                coarse.inv_diag[ci] = fd > T(1e-6) ? T(1) / fd : T(0);
                coarse.px[ci] = px * T(0.5);
                coarse.py[ci] = py * T(0.5);
            }
            w = nw;
        }
    }

    // ---- apply_preconditioner, :1788-1821 (one V-cycle)
    void precondition() {
        size_t start = width, end = start + cells;
        std::fill(base.error.begin() + start, base.error.begin() + end, T(0));
        const T omega = T(1.2);
        base.smooth(false, omega, threads);
        if (!levels.empty()) {
            base.restrict_to(levels[0], threads);
            size_t last = levels.size() - 1;
            for (size_t l = 0; l < last; ++l) {
                levels[l].smooth(false, omega, threads);
                levels[l].restrict_to(levels[l + 1], threads);
            }
            levels[last].solve_coarse_exact();
            for (size_t l = last; l-- > 0;) {
                levels[l].prolongate_from(levels[l + 1], threads);
                levels[l].smooth(true, omega, threads);
            }
            base.prolongate_from(levels[0], threads);
        }
        base.smooth(true, omega, threads);
    }

    // ---- apply_matrix_and_dot, :1823-1863
    T matrix_and_dot(const std::vector<T>& in, std::vector<T>& out) {
        size_t W = width, n = fluid_cells;
        const uint32_t* list = base.fluid.data();
        auto chunk = [&](size_t b, size_t e) -> T {
            T sum = 0;
            for (size_t k = b; k < e; ++k) {
                size_t i = list[k];
                T v = base.diag[i] * in[i];
                v = std::fma(base.px[i], in[i + 1], v);
                v = std::fma(base.px[i - 1], in[i - 1], v);
                v = std::fma(base.py[i], in[i + W], v);
                v = std::fma(base.py[i - W], in[i - W], v);
                out[i] = v;
                sum += v * in[i];
            }
            return sum;
        };
        if (n < 8192) return chunk(0, n);
        size_t nc = (n + 8191) / 8192;
        std::vector<T> parts(nc);
#pragma omp parallel for num_threads(threads) if (par())
        for (size_t c = 0; c < nc; ++c) parts[c] = chunk(c * 8192, std::min(n, (c + 1) * 8192));
        T total = 0;
        for (size_t c = 0; c < nc; ++c) total += parts[c];
        return total;
    }

    // ---- solve_pcg, :1865-1956
    void clear_pressure() {
#pragma omp parallel for num_threads(threads) if (par() && fluid_cells >= 4096)
        for (size_t k = 0; k < fluid_cells; ++k) pressure[base.fluid[k] - width] = T(0);
    }
    void solve_pcg_reference() {
        size_t start = width, end = start + cells;
        clear_pressure();
        stats.pcg_iterations = 0;
        precondition();
        std::copy(base.error.begin() + start, base.error.begin() + end, search.begin() + start);
        T gamma = dot_product(base.residual.data() + start, base.error.data() + start, cells);
        if (gamma < T(1e-5)) { finish_residual_stats(); return; }
        for (int it = 0; it < 100; ++it) {
            T delta = matrix_and_dot(search, ap);
            stats.pcg_iterations++;
            if (std::fabs(delta) < T(1e-5)) break;
            T alpha = gamma / delta;
            T max_err = update_pressure_residual(alpha);
            if (max_err < solve_error) break;
            precondition();
            T ng = dot_product(base.residual.data() + start, base.error.data() + start, cells);
            if (ng < T(1e-5)) break;
            T beta = ng / gamma;
            gamma = ng;
            update_search(beta);
            if (it == 99) stats.not_converged++;
        }
        finish_residual_stats();
    }
    T update_pressure_residual(T alpha) {
        T m = 0;
#pragma omp parallel for num_threads(threads) if (par() && fluid_cells > 4096) reduction(max : m)
        for (size_t k = 0; k < fluid_cells; ++k) {
            size_t pi = base.fluid[k], raw = pi - width;
            pressure[raw] += alpha * search[pi];
            T nr = std::fma(-alpha, ap[pi], base.residual[pi]);
            base.residual[pi] = nr;
            m = std::fmax(m, std::fabs(nr));
        }
        return m;
    }
    void update_search(T beta) {
#pragma omp parallel for num_threads(threads) if (par())
        for (size_t k = 0; k < fluid_cells; ++k) {
            size_t i = base.fluid[k];
            search[i] = base.error[i] + (beta * search[i]);
        }
    }
    double norm2_fluid(const std::vector<T>& v) const {
        double s = 0;
        for (size_t k = 0; k < fluid_cells; ++k) { double x = double(v[base.fluid[k]]); s += x * x; }
        return std::sqrt(s);
    }
    void finish_residual_stats() {
        T m = 0;
        for (size_t k = 0; k < fluid_cells; ++k) m = std::fmax(m, std::fabs(base.residual[base.fluid[k]]));
        stats.residual_max = float(m);
    }

    // FP32 PCG to a relative L2 tolerance (APIC_SOLVER_REL_FP32); also the inner
    // solve of the mixed mode.  The right-hand side is base.residual; the
    // solution is accumulated into `x` (padded layout).  Returns iterations.
    uint32_t pcg_relative(std::vector<T>& x, double tol, uint32_t cap, double* rel_out) {
        size_t start = width, end = start + cells;
        double bnorm = norm2_fluid(base.residual);
        if (rel_out) *rel_out = 0;
        if (bnorm == 0) return 0;
        precondition();
        std::copy(base.error.begin() + start, base.error.begin() + end, search.begin() + start);
        T gamma = dot_product(base.residual.data() + start, base.error.data() + start, cells);
        uint32_t it = 0;
        double rel = 1;
        while (it < cap) {
            T delta = matrix_and_dot(search, ap);
            ++it;
            if (!(delta != T(0)) || !std::isfinite(double(delta))) break;
            T alpha = gamma / delta;
#pragma omp parallel for num_threads(threads) if (par())
            for (size_t k = 0; k < fluid_cells; ++k) {
                size_t pi = base.fluid[k];
                x[pi] += alpha * search[pi];
                base.residual[pi] = std::fma(-alpha, ap[pi], base.residual[pi]);
            }
            rel = norm2_fluid(base.residual) / bnorm;
            if (rel <= tol) break;
            precondition();
            T ng = dot_product(base.residual.data() + start, base.error.data() + start, cells);
            if (!(ng != T(0))) break;
            T beta = ng / gamma;
            gamma = ng;
            update_search(beta);
        }
        if (rel_out) *rel_out = rel;
        return it;
    }

    // True residual ||b - A p|| / ||b|| in FP64 over the fluid cells.
    double true_residual(const std::vector<double>& b, const std::vector<double>& p, std::vector<double>* r) const {
        size_t W = width;
        double rn = 0, bn = 0;
        for (size_t k = 0; k < fluid_cells; ++k) {
            size_t i = base.fluid[k];
            double v = double(base.diag[i]) * p[i] + double(base.px[i]) * p[i + 1] + double(base.px[i - 1]) * p[i - 1] +
                       double(base.py[i]) * p[i + W] + double(base.py[i - W]) * p[i - W];
            double ri = b[i] - v;
            if (r) (*r)[i] = ri;
            rn += ri * ri;
            bn += b[i] * b[i];
        }
        return bn > 0 ? std::sqrt(rn / bn) : 0.0;
    }

    void solve_pcg_relative(bool mixed) {
        size_t n = base.residual.size();
        clear_pressure();
        stats.pcg_iterations = 0;
        stats.refinement_steps = 0;
        std::vector<double> b(n, 0.0), p64(n, 0.0), r64(n, 0.0);
        if (mixed && warm_start && this->p64.size() == n) p64 = this->p64;
        for (size_t k = 0; k < fluid_cells; ++k) b[base.fluid[k]] = double(base.residual[base.fluid[k]]);
        std::vector<T> x(n, T(0));
        double rel = 0;
        if (!mixed) {
            uint32_t it = pcg_relative(x, double(rel_tol), max_iter, &rel);
            stats.pcg_iterations = it;
            if (rel > double(rel_tol)) stats.not_converged++;
            for (size_t k = 0; k < fluid_cells; ++k) p64[base.fluid[k]] = double(x[base.fluid[k]]);
        } else {
            // Each inner solve reduces its right-hand side (the current true
            // residual) by 1e-4, or to rel_tol / 2 of ||b|| when that comes first.
            uint32_t used = 0;
            const double inner_reduction = 1e-4;
            for (int outer = 0; outer < 32 && used < max_iter; ++outer) {
                double tr = true_residual(b, p64, &r64);
                if (tr <= double(rel_tol)) break;
                stats.refinement_steps++;
                for (size_t k = 0; k < fluid_cells; ++k) {
                    size_t i = base.fluid[k];
                    base.residual[i] = T(r64[i]);
                    x[i] = T(0);
                }
                double irel = 0;
                double target = std::max(inner_reduction, 0.5 * double(rel_tol) / std::max(tr, 1e-300));
                used += pcg_relative(x, target, max_iter - used, &irel);
                for (size_t k = 0; k < fluid_cells; ++k) p64[base.fluid[k]] += double(x[base.fluid[k]]);
            }
            stats.pcg_iterations = used;
        }
        for (size_t k = 0; k < fluid_cells; ++k) {
            size_t i = base.fluid[k];
            pressure[i - width] = T(p64[i]);
        }
        // the mixed mode projects with the FP64 pressure; the plain mode with the FP32 one
        std::vector<double> pf(n, 0.0);
        if (mixed) pf = p64;
        else
            for (size_t k = 0; k < fluid_cells; ++k) pf[base.fluid[k]] = double(pressure[base.fluid[k] - width]);
        if (mixed) { this->p64 = p64; p64_valid = true; }
        double tr = true_residual(b, pf, &r64);
        stats.true_residual_rel = tr;
        if (mixed && tr > double(rel_tol)) stats.not_converged++;
        for (size_t k = 0; k < fluid_cells; ++k) base.residual[base.fluid[k]] = T(r64[base.fluid[k]]);
        finish_residual_stats();
        double bn = 0;
        for (size_t k = 0; k < fluid_cells; ++k) bn += b[base.fluid[k]] * b[base.fluid[k]];
        stats.residual_rel = float(bn > 0 ? norm2_fluid(base.residual) / std::sqrt(bn) : 0.0);
    }

    void solve() {
        p64_valid = false;
        if (solver_mode == APIC_SOLVER_REFERENCE) solve_pcg_reference();
        else solve_pcg_relative(solver_mode == APIC_SOLVER_REL_MIXED);
        stats.pcg_iterations_total += stats.pcg_iterations;
    }

    // ---- apply_pressure_gradient, :1958-2055
    void pressure_gradient() {
        const T target = T(9.0);
        const T inv = T(1) / cell_size;
        const int32_t W = int32_t(width), H = int32_t(height);
#pragma omp parallel for num_threads(threads) if (par())
        for (int32_t y = 0; y < H; ++y)
            for (int32_t x = 0; x <= W; ++x) {
                size_t f = u_index(x, y);
                int32_t lx = x - 1;
                bool lo = is_obstacle(lx, y) == 1, ro = is_obstacle(x, y) == 1;
                if (lo != ro) { mac_u[f] = T(0); valid_u[f] = 1; continue; }
                bool lf = is_fluid(lx, y) == 1, rf = is_fluid(x, y) == 1;
                T dp = 0;
                size_t li = size_t(y * W + lx), ri = size_t(y * W + x);
                if (p64_valid) {  // mixed mode: FP64 pressure differences
                    double d = 0.0;
                    if (lf && rf) d = p64[ri + W] - p64[li + W];
                    else if (lf) d = -p64[li + W] / double(theta(smoothed[ri], smoothed[li], target));
                    else if (rf) d = p64[ri + W] / double(theta(smoothed[li], smoothed[ri], target));
                    mac_u[f] -= T(d * double(inv));
                    continue;
                }
                if (lf && rf) dp = pressure[ri] - pressure[li];
                else if (lf) { T th = theta(smoothed[ri], smoothed[li], target); dp = -pressure[li] / th; }
                else if (rf) { T th = theta(smoothed[li], smoothed[ri], target); dp = pressure[ri] / th; }
                mac_u[f] -= dp * inv;
            }
#pragma omp parallel for num_threads(threads) if (par())
        for (int32_t y = 0; y <= H; ++y)
            for (int32_t x = 0; x < W; ++x) {
                size_t f = v_index(x, y);
                int32_t by = y - 1;
                bool bo = is_obstacle(x, by) == 1, to = is_obstacle(x, y) == 1;
                if (bo != to) { mac_v[f] = T(0); valid_v[f] = 1; continue; }
                bool bf = is_fluid(x, by) == 1, tf = is_fluid(x, y) == 1;
                T dp = 0;
                size_t bi = size_t(by * W + x), ti = size_t(y * W + x);
                if (p64_valid) {
                    double d = 0.0;
                    if (bf && tf) d = p64[ti + W] - p64[bi + W];
                    else if (bf) d = -p64[bi + W] / double(theta(smoothed[ti], smoothed[bi], target));
                    else if (tf) d = p64[ti + W] / double(theta(smoothed[bi], smoothed[ti], target));
                    mac_v[f] -= T(d * double(inv));
                    continue;
                }
                if (bf && tf) dp = pressure[ti] - pressure[bi];
                else if (bf) { T th = theta(smoothed[ti], smoothed[bi], target); dp = -pressure[bi] / th; }
                else if (tf) { T th = theta(smoothed[bi], smoothed[ti], target); dp = pressure[ti] / th; }
                mac_v[f] -= dp * inv;
            }
    }

    // ---- post forces, :2453-2458
    void post_forces(T dt) {
        for (size_t i = 0; i < mac_u.size(); ++i) mac_u[i] += post_u[i] * dt;
        for (size_t i = 0; i < mac_v.size(); ++i) mac_v[i] += post_v[i] * dt;
    }

    // ---- extrapolate_velocity, :2266-2350
    void extrapolate() {
        const size_t W = width, H = height;
        for (int s = 0; s < 4; ++s) {
            std::swap(mac_u, old_u);
            std::swap(valid_u, next_valid_u);
#pragma omp parallel for num_threads(threads) if (par())
            for (size_t y = 0; y < H; ++y)
                for (size_t x = 0; x <= W; ++x) {
                    size_t i = y * (W + 1) + x;
                    if (next_valid_u[i]) { mac_u[i] = old_u[i]; valid_u[i] = 1; continue; }
                    T sum = 0; uint32_t cnt = 0;
                    if (x > 0 && next_valid_u[i - 1]) { sum += old_u[i - 1]; cnt++; }
                    if (x < W && next_valid_u[i + 1]) { sum += old_u[i + 1]; cnt++; }
                    if (y > 0 && next_valid_u[i - (W + 1)]) { sum += old_u[i - (W + 1)]; cnt++; }
                    if (y < H - 1 && next_valid_u[i + W + 1]) { sum += old_u[i + W + 1]; cnt++; }
                    if (cnt > 0) { mac_u[i] = sum / T(cnt); valid_u[i] = 1; }
                    else { mac_u[i] = old_u[i]; valid_u[i] = 0; }
                }
        }
        for (int s = 0; s < 4; ++s) {
            std::swap(mac_v, old_v);
            std::swap(valid_v, next_valid_v);
#pragma omp parallel for num_threads(threads) if (par())
            for (size_t y = 0; y <= H; ++y)
                for (size_t x = 0; x < W; ++x) {
                    size_t i = y * W + x;
                    if (next_valid_v[i]) { mac_v[i] = old_v[i]; valid_v[i] = 1; continue; }
                    T sum = 0; uint32_t cnt = 0;
                    if (x > 0 && next_valid_v[i - 1]) { sum += old_v[i - 1]; cnt++; }
                    if (x < W - 1 && next_valid_v[i + 1]) { sum += old_v[i + 1]; cnt++; }
                    if (y > 0 && next_valid_v[i - W]) { sum += old_v[i - W]; cnt++; }
                    if (y < H && next_valid_v[i + W]) { sum += old_v[i + W]; cnt++; }
                    if (cnt > 0) { mac_v[i] = sum / T(cnt); valid_v[i] = 1; }
                    else { mac_v[i] = old_v[i]; valid_v[i] = 0; }
                }
        }
    }

    // ---- transfer_grid_to_particles_and_advect, :2057-2264 (all padded lanes)
    static T bilinear(const T w[4], const T v[4]) {  // :138-172
        T ws = w[0] + w[1] + w[2] + w[3];
        T inv = T(1.0) / fmax_x86(ws, T(1e-6));
        T vel = 0;
        for (int k = 0; k < 4; ++k) vel += v[k] * w[k] * inv;
        return vel;
    }
    static bool bit(const std::vector<uint64_t>& m, uint32_t i) { return (m[i >> 6] >> (i & 63)) & 1; }

    void g2p(T dt) {
        const T cs = cell_size;
        const T min_x = T(1.001) * cs, max_x = (T(width) - T(1.001)) * cs;
        const T min_y = T(1.001) * cs, max_y = (T(height) - T(1.001)) * cs;
        const T h2 = cs * cs, one = T(1), eps = T(1e-6), zero = T(0);
        const T bd = -border_damping;
        const uint32_t ts = timestamp;
        const size_t n = npad();
        uint32_t nonfinite = 0;
#pragma omp parallel for num_threads(threads) if (par()) reduction(+ : nonfinite)
        for (size_t i = 0; i < n; ++i) {
            T px = part[PX][i], py = part[PY][i];
            T gx = px / cs, gy = py / cs;
            Stencil su, sv;
            u_stencil(gx, gy, su);
            v_stencil(gx, gy, sv);
            T un[4], vn[4], uwm[4], vwm[4];
            for (int k = 0; k < 4; ++k) {
                un[k] = mac_u[su.idx[k]]; vn[k] = mac_v[sv.idx[k]];
                uwm[k] = bit(u_open, su.idx[k]) ? su.w[k] : T(0);
                vwm[k] = bit(v_open, sv.idx[k]) ? sv.w[k] : T(0);
            }
            T nvx = bilinear(uwm, un), nvy = bilinear(vwm, vn);
            T res = part[TR][i];
            T speed = std::sqrt(nvx * nvx + nvy * nvy);
            T cfl_local = speed * dt / cs;
            T scale = fmin_x86(fmax_x86(cfl_local, zero), T(1.0));
            T gam = scale * scale * (T(3.0) - (T(2.0) * scale));
            T jitter = gam * T(random_lane(uint32_t(i), ts)) * dt;
            T dt_raw = dt + res + jitter;
            T dt_act = fmin_x86(fmax_x86(dt_raw, zero), dt * T(2.0));
            part[TR][i] = dt + res - dt_act;
            T nx = px + dt_act * nvx, ny = py + dt_act * nvy;
            bool oxmin = nx < min_x, oxmax = nx > max_x, oymin = ny < min_y, oymax = ny > max_y;
            bool ovxmin = oxmin && nvx < zero, ovxmax = oxmax && nvx > zero;
            bool ovymin = oymin && nvy < zero, ovymax = oymax && nvy > zero;
            if (oxmin) nx = min_x;
            if (oxmax) nx = max_x;
            if (ovxmin) nvx = nvx * bd;
            if (ovxmax) nvx = nvx * bd;
            if (oymin) ny = min_y;
            if (oymax) ny = max_y;
            if (ovymin) nvy = nvy * bd;
            if (ovymax) nvy = nvy * bd;
            T udx = h2 * su.tx * (one - su.tx), udy = h2 * su.ty * (one - su.ty);
            T vdx = h2 * sv.tx * (one - sv.tx), vdy = h2 * sv.ty * (one - sv.ty);
            T uix = udx > eps ? one / udx : zero, uiy = udy > eps ? one / udy : zero;
            T vix = vdx > eps ? one / vdx : zero, viy = vdy > eps ? one / vdy : zero;
            T cux = 0, cuy = 0, cvx = 0, cvy = 0;
            for (int k = 0; k < 4; ++k) {
                cux += su.w[k] * un[k] * su.dx[k];
                cuy += su.w[k] * un[k] * su.dy[k];
            }
            for (int k = 0; k < 4; ++k) {
                cvx += sv.w[k] * vn[k] * sv.dx[k];
                cvy += sv.w[k] * vn[k] * sv.dy[k];
            }
            T cu_x = cux * uix, cu_y = cuy * uiy, cv_x = cvx * vix, cv_y = cvy * viy;
            bool rx = ovxmin || ovxmax, ry = ovymin || ovymax;
            if (rx) { cu_y = cu_y * T(-1.0); cv_x = cv_x * T(-1.0); }
            if (ry) { cu_y = cu_y * T(-1.0); cv_x = cv_x * T(-1.0); }
            part[PX][i] = nx; part[PY][i] = ny; part[VX][i] = nvx; part[VY][i] = nvy;
            part[CUX][i] = cu_x; part[CUY][i] = cu_y; part[CVX][i] = cv_x; part[CVY][i] = cv_y;
            if (!std::isfinite(double(nx)) || !std::isfinite(double(ny))) nonfinite++;
        }
        stats.nonfinite_lanes = nonfinite;
    }

    // ---- add_radial_force, :2352-2410
    void add_radial_force(T wx, T wy, T radius, T strength) {
        uint32_t mnx = uint32_t(std::max(int32_t(std::floor((wx - radius) / cell_size)), 0));
        uint32_t mxx = uint32_t(std::min(int32_t(std::ceil((wx + radius) / cell_size)), int32_t(width)));
        uint32_t mny = uint32_t(std::max(int32_t(std::floor((wy - radius) / cell_size)), 0));
        uint32_t mxy = uint32_t(std::min(int32_t(std::ceil((wy + radius) / cell_size)), int32_t(height)));
        T r2 = radius * radius;
        bool repel = strength > T(0);
        for (uint32_t y = mny; y <= mxy; ++y)
            for (uint32_t x = mnx; x <= mxx; ++x) {
                if (x <= width && y < height) {
                    T dx = T(x) * cell_size - wx, dy = (T(y) + T(0.5)) * cell_size - wy;
                    T d2 = dx * dx + dy * dy;
                    if (d2 < r2 && d2 > T(1e-5)) {
                        T d = std::sqrt(d2);
                        T fall = T(1) - (d / radius);
                        T force = (dx / d) * strength * fall;
                        size_t ui = u_index(int32_t(x), int32_t(y));
                        (repel ? post_u : ext_u)[ui] += force;
                    }
                }
                if (x < width && y <= height) {
                    T dx = (T(x) + T(0.5)) * cell_size - wx, dy = T(y) * cell_size - wy;
                    T d2 = dx * dx + dy * dy;
                    if (d2 < r2 && d2 > T(1e-5)) {
                        T d = std::sqrt(d2);
                        T fall = T(1) - (d / radius);
                        T force = (dy / d) * strength * fall;
                        size_t vi = v_index(int32_t(x), int32_t(y));
                        (repel ? post_v : ext_v)[vi] += force;
                    }
                }
            }
    }

    // ---- Apic::update, :2429-2474
    int update(uint32_t flags, T frame_dt) {
        T t = 0;
        stats.substeps = 0;
        stats.pcg_iterations_total = 0;
        stats.not_converged = 0;
        while (t < frame_dt) {
            T vmax = max_particle_velocity();
            T safe = vmax > T(1e-5) ? cfl * cell_size / vmax : frame_dt;
            T step = std::fmin(safe, frame_dt - t);
            if (!(step > T(0)) || stats.substeps >= 100000) return APIC_ERR_NONFINITE;  // the reference loops forever here
            if (!(flags & APIC_UPDATE_DISABLE_SORT) && t == T(0)) spatial_lookup();
            substep(step);
            t += step;
            prev_dt = step;
            timestamp += 1;
            stats.substeps++;
        }
        std::fill(ext_u.begin(), ext_u.end(), T(0)); std::fill(ext_v.begin(), ext_v.end(), T(0));
        std::fill(post_u.begin(), post_u.end(), T(0)); std::fill(post_v.begin(), post_v.end(), T(0));
        return APIC_OK;
    }
    void substep(T step) {
        p2g();
        external_forces(step);
        build_pressure();
        update_multilevel();
        solve();
        pressure_gradient();
        post_forces(step);
        extrapolate();
        g2p(step);
    }

    int run_stage(int stage, T dt) {
        switch (stage) {
            case APIC_STAGE_SORT: spatial_lookup(); break;
            case APIC_STAGE_P2G: p2g(); break;
            case APIC_STAGE_FORCES: external_forces(dt); break;
            case APIC_STAGE_BUILD: build_pressure(); break;
            case APIC_STAGE_MG: update_multilevel(); break;
            case APIC_STAGE_PCG: stats.pcg_iterations_total = 0; solve(); break;
            case APIC_STAGE_GRAD: pressure_gradient(); break;
            case APIC_STAGE_POST: post_forces(dt); break;
            case APIC_STAGE_EXTRAP: extrapolate(); break;
            case APIC_STAGE_G2P: g2p(dt); break;
            case APIC_STAGE_VMAX: break;
            case APIC_STAGE_VCYCLE: precondition(); break;
            default: return APIC_ERR_INVALID_ARG;
        }
        return APIC_OK;
    }

    // ---- field access
    struct FieldRef {
        void* ptr = nullptr;
        uint64_t count = 0;
        uint32_t elem = 0;
        int kind = 0;  // 0 = T, 1 = u8, 2 = u64, 3 = u32
    };
    template <class V> FieldRef ref_of(std::vector<V>& v, uint64_t count, int kind) {
        FieldRef r;
        r.ptr = v.data();
        r.count = count;
        r.elem = uint32_t(sizeof(V));
        r.kind = kind;
        return r;
    }
    bool field(int id, FieldRef& r) {
        size_t padded = size_t(cells) + 2 * size_t(width);
        if (id >= APIC_F_POS_X && id <= APIC_F_TRES) { r = ref_of(part[id], npad(), 0); return true; }
        switch (id) {
            case APIC_F_U: r = ref_of(mac_u, u_faces(), 0); return true;
            case APIC_F_V: r = ref_of(mac_v, v_faces(), 0); return true;
            case APIC_F_VALID_U: r = ref_of(valid_u, u_faces(), 1); return true;
            case APIC_F_VALID_V: r = ref_of(valid_v, v_faces(), 1); return true;
            case APIC_F_DENSITY: r = ref_of(density, cells, 0); return true;
            case APIC_F_SMOOTHED_DENSITY: r = ref_of(smoothed, cells, 0); return true;
            case APIC_F_PRESSURE: r = ref_of(pressure, cells, 0); return true;
            case APIC_F_FLUID_BITS: r = ref_of(base.fluid_bits, base.fluid_bits.size(), 2); return true;
            case APIC_F_OBSTACLE_BITS: r = ref_of(obstacle, obstacle.size(), 2); return true;
            case APIC_F_U_OPEN_BITS: r = ref_of(u_open, u_open.size(), 2); return true;
            case APIC_F_V_OPEN_BITS: r = ref_of(v_open, v_open.size(), 2); return true;
            case APIC_F_RESIDUAL: r = ref_of(base.residual, padded, 0); return true;
            case APIC_F_DIAG: r = ref_of(base.diag, padded, 0); return true;
            case APIC_F_INV_DIAG: r = ref_of(base.inv_diag, padded, 0); return true;
            case APIC_F_PLUS_X: r = ref_of(base.px, padded, 0); return true;
            case APIC_F_PLUS_Y: r = ref_of(base.py, padded, 0); return true;
            case APIC_F_ERROR: r = ref_of(base.error, padded, 0); return true;
            case APIC_F_SORT_KEYS: r = ref_of(sort_key, sort_key.size(), 3); return true;
            case APIC_F_SORT_VALS: r = ref_of(sort_val, sort_val.size(), 3); return true;
            case APIC_F_FLUID_LIST: r = ref_of(base.fluid, fluid_cells, 3); return true;
            case APIC_F_EXT_FORCE_U: r = ref_of(ext_u, u_faces(), 0); return true;
            case APIC_F_EXT_FORCE_V: r = ref_of(ext_v, v_faces(), 0); return true;
            case APIC_F_POST_FORCE_U: r = ref_of(post_u, u_faces(), 0); return true;
            case APIC_F_POST_FORCE_V: r = ref_of(post_v, v_faces(), 0); return true;
            default: break;
        }
        if (id >= APIC_F_MG_FLUID_BITS) {
            int l = id / APIC_F_MG_LEVEL_STRIDE;
            int f = id % APIC_F_MG_LEVEL_STRIDE;
            if (l < 0 || size_t(l) >= levels.size()) return false;
            Level<T>& L = levels[size_t(l)];
            size_t lp = L.cells + 2 * L.width;
            switch (f) {
                case APIC_F_MG_FLUID_BITS: r = ref_of(L.fluid_bits, L.fluid_bits.size(), 2); return true;
                case APIC_F_MG_DIAG: r = ref_of(L.diag, lp, 0); return true;
                case APIC_F_MG_INV_DIAG: r = ref_of(L.inv_diag, lp, 0); return true;
                case APIC_F_MG_PLUS_X: r = ref_of(L.px, lp, 0); return true;
                case APIC_F_MG_PLUS_Y: r = ref_of(L.py, lp, 0); return true;
                default: return false;
            }
        }
        return false;
    }

    // After a write of a mask field, rebuild the lists that the reference keeps
    // beside it (fluid/red/black lists and the padded list, :1461-1494).
    void rebuild_base_lists() {
        base.fluid.clear(); base.red.clear(); base.black.clear();
        fluid_cells = 0;
        for (size_t i = 0; i < base.fluid_bits.size(); ++i) {
            uint64_t m = base.fluid_bits[i];
            while (m) {
                size_t raw = i * 64 + size_t(__builtin_ctzll(m));
                uint32_t padded = uint32_t(raw + width);
                base.fluid.push_back(padded);
                ++fluid_cells;
                size_t x = raw % width, y = raw / width;
                ((x + y) % 2 == 0 ? base.red : base.black).push_back(padded);
                m &= m - 1;
            }
        }
        uint32_t rem = fluid_cells % 8;
        if (rem) {
            uint32_t last = base.fluid[fluid_cells - 1];
            for (uint32_t k = 0; k < 8 - rem; ++k) base.fluid.push_back(last);
        }
    }
};

struct Handle {
    int fp64 = 0;
    std::unique_ptr<Sim<float>> f;
    std::unique_ptr<Sim<double>> d;
};

template <class F> int dispatch(oracle_sim* o, F&& fn) {
    if (!o) return APIC_ERR_INVALID_ARG;
    Handle* h = reinterpret_cast<Handle*>(o);
    if (h->fp64) return fn(*h->d);
    return fn(*h->f);
}

}  // namespace

extern "C" {

oracle_sim* oracle_create(uint32_t width, uint32_t height, float cell_size, const apic_world_props* props,
                          int fp64, int threads) {
    if (!props || width == 0 || height == 0) return nullptr;
    Handle* h = new Handle();
    h->fp64 = fp64 ? 1 : 0;
    if (h->fp64) { h->d.reset(new Sim<double>()); h->d->threads = threads; h->d->construct(width, height, cell_size, *props); }
    else { h->f.reset(new Sim<float>()); h->f->threads = threads; h->f->construct(width, height, cell_size, *props); }
    return reinterpret_cast<oracle_sim*>(h);
}

void oracle_destroy(oracle_sim* o) { delete reinterpret_cast<Handle*>(o); }

int oracle_set_threads(oracle_sim* o, int threads) {
    return dispatch(o, [&](auto& s) { s.threads = threads; return APIC_OK; });
}

int oracle_set_particles(oracle_sim* o, uint32_t n, const float* px, const float* py, const float* vx, const float* vy) {
    return dispatch(o, [&](auto& s) {
        using T = typename std::remove_reference<decltype(s.cell_size)>::type;
        if (n > 0 && (!px || !py)) return APIC_ERR_INVALID_ARG;
        s.p64.clear();  // a new particle set: the next mixed solve starts from zero
        s.p64_valid = false;
        std::vector<T> ix(n), iy(n), ivx(n, T(0)), ivy(n, T(0));
        for (uint32_t i = 0; i < n; ++i) {
            ix[i] = T(px[i]); iy[i] = T(py[i]);
            if (vx) ivx[i] = T(vx[i]);
            if (vy) ivy[i] = T(vy[i]);
        }
        if (n == 0) {
            s.num_particles = 0; s.num_chunks = 0;
            for (int f = 0; f < s.NPF; ++f) { s.part[f].clear(); s.part_sort[f].clear(); }
            s.sort_key.clear(); s.sort_val.clear();
            return APIC_OK;
        }
        if (s.levels.empty() && !s.build_levels()) return APIC_ERR_INVALID_ARG;
        s.load_positions(ix, iy, &ivx, &ivy);
        if (!s.world_ready) s.update_world();
        return APIC_OK;
    });
}

int oracle_set_warm_start(oracle_sim* o, int enabled) {
    return dispatch(o, [&](auto& s) {
        s.warm_start = enabled != 0;
        return APIC_OK;
    });
}

int oracle_set_solver(oracle_sim* o, int mode, float rel_tol, uint32_t max_iterations) {
    return dispatch(o, [&](auto& s) {
        if (mode < 0 || mode > 2) return APIC_ERR_INVALID_ARG;
        s.solver_mode = mode;
        s.rel_tol = rel_tol;
        s.max_iter = max_iterations;
        return APIC_OK;
    });
}

int oracle_update(oracle_sim* o, uint32_t flags, float frame_dt) {
    return dispatch(o, [&](auto& s) { return s.update(flags, frame_dt); });
}

int oracle_run_stage(oracle_sim* o, int stage, float dt) {
    return dispatch(o, [&](auto& s) { return s.run_stage(stage, dt); });
}

int oracle_finish_substep(oracle_sim* o, float dt) {
    return dispatch(o, [&](auto& s) {
        s.prev_dt = dt;
        s.timestamp += 1;
        return APIC_OK;
    });
}

int oracle_max_particle_velocity(oracle_sim* o, float* out) {
    return dispatch(o, [&](auto& s) { *out = float(s.max_particle_velocity()); return APIC_OK; });
}

int oracle_add_radial_force(oracle_sim* o, float x, float y, float radius, float strength) {
    return dispatch(o, [&](auto& s) { s.add_radial_force(x, y, radius, strength); return APIC_OK; });
}

int oracle_get_info(oracle_sim* o, apic_info* out) {
    return dispatch(o, [&](auto& s) {
        out->width = s.width; out->height = s.height; out->cells = s.cells;
        out->cell_size = float(s.cell_size);
        out->num_chunks = s.num_chunks; out->num_particles = s.num_particles;
        out->fluid_cells = s.fluid_cells; out->timestamp = s.timestamp;
        out->prev_deltatime = float(s.prev_dt);
        out->mg_levels = uint32_t(s.levels.size());
        return APIC_OK;
    });
}

int oracle_get_stats(oracle_sim* o, apic_step_stats* out) {
    return dispatch(o, [&](auto& s) { *out = s.stats; return APIC_OK; });
}

int oracle_field_shape(oracle_sim* o, int field, uint64_t* count, uint32_t* elem_bytes) {
    return dispatch(o, [&](auto& s) {
        typename std::remove_reference<decltype(s)>::type::FieldRef r;
        if (!s.field(field, r)) return APIC_ERR_INVALID_ARG;
        *count = r.count;
        *elem_bytes = r.elem;
        return APIC_OK;
    });
}

int oracle_read_field(oracle_sim* o, int field, void* dst, uint64_t bytes) {
    return dispatch(o, [&](auto& s) {
        typename std::remove_reference<decltype(s)>::type::FieldRef r;
        if (!s.field(field, r)) return APIC_ERR_INVALID_ARG;
        if (bytes != r.count * r.elem) return APIC_ERR_INVALID_ARG;
        if (bytes) std::memcpy(dst, r.ptr, bytes);
        return APIC_OK;
    });
}

int oracle_write_field(oracle_sim* o, int field, const void* src, uint64_t bytes) {
    return dispatch(o, [&](auto& s) {
        typename std::remove_reference<decltype(s)>::type::FieldRef r;
        if (!s.field(field, r)) return APIC_ERR_INVALID_ARG;
        if (bytes != r.count * r.elem) return APIC_ERR_INVALID_ARG;
        if (field == APIC_F_SORT_KEYS || field == APIC_F_SORT_VALS || field == APIC_F_FLUID_LIST)
            return APIC_ERR_INVALID_ARG;
        if (bytes) std::memcpy(r.ptr, src, bytes);
        if (field == APIC_F_PRESSURE) s.p64_valid = false;
        if (field == APIC_F_FLUID_BITS) s.rebuild_base_lists();
        if (field == APIC_F_OBSTACLE_BITS) s.update_world();
        return APIC_OK;
    });
}

// ---- headless particle view ----------------------------------------------
// render_particles (src/main.rs:207-277) as a sequential loop over the
// particles in index order, each drawn as a textured quad into an RGBA8
// frame: texture of make_circle_texture (:73-101), bilinear clamp-to-edge
// sampling with texel centres at (i + 0.5) / 32 (texel coordinate
// (pixel centre - quad corner) * (32 / 2R) - 0.5), a pixel covered when its
// centre lies in [x0, x0 + 2R), blend src*a + dst*(1 - a) rounded to 8 bits
// after every particle.
static uint8_t circle_alpha(int x, int y) {
    const float radius = 32.0f / 2.0f;
    const float dx = float(x) - radius + 0.5f;
    const float dy = float(y) - radius + 0.5f;
    const float dist = std::sqrt(dx * dx + dy * dy);
    if (dist < radius - 1.0f) return 255;
    if (dist < radius) {
        const float a = (radius - dist) * 255.0f;  // Rust `as u8` saturates
        return a >= 255.0f ? 255 : (a > 0.0f ? uint8_t(a) : 0);
    }
    return 0;
}

static uint8_t blend8(float c, float a, uint8_t dst) {
    const float d = float(dst) / 255.0f;
    const float o = c * a + d * (1.0f - a);
    const float q = o * 255.0f + 0.5f;
    return q >= 255.0f ? 255 : (q > 0.0f ? uint8_t(q) : 0);
}

int oracle_render(uint32_t n, const float* px, const float* py, const float* vx, const float* vy,
                  const apic_render_params* rp, uint32_t fluid_cells, float cell_size, uint8_t* rgba,
                  apic_render_stats* st) {
    if (!rp || !rgba || !st || (n && (!px || !py || !vx || !vy))) return APIC_ERR_INVALID_ARG;
    const apic_render_params& p = *rp;
    const uint32_t W = p.width, H = p.height;
    float tex[32 * 32];
    for (int y = 0; y < 32; ++y)
        for (int x = 0; x < 32; ++x) tex[y * 32 + x] = float(circle_alpha(x, y)) / 255.0f;
    for (uint64_t i = 0; i < uint64_t(W) * H; ++i) {
        rgba[i * 4 + 0] = uint8_t(p.background & 0xFFu);
        rgba[i * 4 + 1] = uint8_t((p.background >> 8) & 0xFFu);
        rgba[i * 4 + 2] = uint8_t((p.background >> 16) & 0xFFu);
        rgba[i * 4 + 3] = 255;
    }
    const float fw = float(W), fh = float(H);
    const float R = p.draw_radius, S = p.draw_radius * 2.0f;
    const float tex_scale = 32.0f / S;  // texels per pixel
    const float pick_r2 = p.pick_radius < 0.0f ? -1.0f : p.pick_radius * p.pick_radius;
    float best = INFINITY;
    int64_t picked = -1;
    uint32_t valid = 0, nan = 0, oob = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const float x = px[i], y = py[i];
        if (!std::isfinite(x) || !std::isfinite(y)) {
            ++nan;
            continue;
        }
        const float draw_x = x * p.scale;
        const float draw_y = fh - y * p.scale;
        if (draw_x < -p.margin || draw_x > fw + p.margin || draw_y < -p.margin || draw_y > fh + p.margin) {
            ++oob;
            continue;
        }
        ++valid;
        if (pick_r2 >= 0.0f) {
            const float dx = draw_x - p.pick_x;
            const float dy = draw_y - p.pick_y;
            const float d2 = dx * dx + dy * dy;
            if (d2 <= pick_r2 && d2 < best) {
                best = d2;
                picked = i;
            }
        }
        const float speed_sq = vx[i] * vx[i] + vy[i] * vy[i];
        const float r = std::fmin(speed_sq * 0.01f, 1.0f);  // f32::min ignores a NaN operand, as fmin does
        const float g = 0.5f, b = 1.0f - r * 0.5f;
        const float qx = draw_x - R, qy = draw_y - R;
        // pixels whose centres can lie in [q, q + S): a window one pixel wider
        const long x_lo = std::max(0L, long(std::floor(qx)) - 1), x_hi = std::min(long(W) - 1, long(std::floor(qx + S)) + 1);
        const long y_lo = std::max(0L, long(std::floor(qy)) - 1), y_hi = std::min(long(H) - 1, long(std::floor(qy + S)) + 1);
        for (long pyi = y_lo; pyi <= y_hi; ++pyi)
            for (long pxi = x_lo; pxi <= x_hi; ++pxi) {
                const float cx = float(pxi) + 0.5f, cy = float(pyi) + 0.5f;
                if (!(qx <= cx && cx < qx + S && qy <= cy && cy < qy + S)) continue;
                const float u = (cx - qx) * tex_scale - 0.5f;
                const float v = (cy - qy) * tex_scale - 0.5f;
                const float fu = std::floor(u), fv = std::floor(v);
                const float wu = u - fu, wv = v - fv;
                const int iu = int(fu), iv = int(fv);
                const int u0 = std::min(std::max(iu, 0), 31), u1 = std::min(std::max(iu + 1, 0), 31);
                const int v0 = std::min(std::max(iv, 0), 31), v1 = std::min(std::max(iv + 1, 0), 31);
                const float top = tex[v0 * 32 + u0] * (1.0f - wu) + tex[v0 * 32 + u1] * wu;
                const float bot = tex[v1 * 32 + u0] * (1.0f - wu) + tex[v1 * 32 + u1] * wu;
                const float a = top * (1.0f - wv) + bot * wv;
                uint8_t* d = rgba + (uint64_t(pyi) * W + uint64_t(pxi)) * 4;
                d[0] = blend8(r, a, d[0]);
                d[1] = blend8(g, a, d[1]);
                d[2] = blend8(b, a, d[2]);
            }
    }
    st->valid = valid;
    st->nan = nan;
    st->out_of_bounds = oob;
    st->fluid_cells = fluid_cells;
    st->picked = picked;
    st->volume = float(fluid_cells) * (cell_size * cell_size);
    st->kernels = 0;
    return APIC_OK;
}

uint32_t oracle_morton(uint32_t x, uint32_t y) { return morton(x, y); }
float oracle_random_lane(uint32_t slot, uint32_t seed) { return random_lane(slot, seed); }
float oracle_temporal_weight(float tau) { return temporal_w(tau); }

}  // extern "C"
