// scene.cpp — deterministic particle scenes for the benchmark configurations.
//
// Host code only (no GPU).  Every random number comes from the reference's
// own 32-bit mixing hash (the lowbias32-style mixer of Apic::random_simd,
// src/apic.rs:960-966) keyed by (seed, stream, particle or lattice id), so the
// same parameters give bit-identical particles on every machine.  Gaussian
// velocities use Box-Muller in double precision, rounded to float.
//
// Scenes (cells on the one-cell solid border never receive particles, as in
// Apic::new, src/apic.rs:831-849):
//   REFERENCE_DEFAULT  Apic::new's block: 3 x 3 particles per cell for
//                      4 < x < W-4, 4 < y < H/2 at sub-cell centres.
//   DAM_BREAK          cells whose centre has x < fluid_x and y < fluid_y,
//                      sub x sub particles per cell, each jittered uniformly
//                      inside its sub-cell.
//   DAM_BREAK_DISK     the dam break plus cells whose centre lies within
//                      disk_r of (disk_x, disk_y), moving at (disk_vx, disk_vy).
//   NOISE              cells where a value noise (hash-valued lattice of period
//                      noise_period, smoothstep-interpolated) exceeds
//                      noise_threshold; velocities N(0, vel_sigma^2) per component.
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/apic_gpu.h"

namespace {

inline uint32_t mix32(uint32_t m) {
    m ^= m >> 16;
    m *= 0x7feb352du;
    m ^= m >> 15;
    m *= 0x846ca68bu;
    m ^= m >> 16;
    return m;
}

inline uint32_t stream_key(uint32_t seed, uint32_t stream) { return mix32(seed * 0x9E3779B9u ^ mix32(stream + 0x632BE5ABu)); }

// Uniform in [0, 1) with 24 random bits.
inline double u01(uint32_t key, uint32_t id) { return double(mix32(id ^ key) >> 8) * (1.0 / 16777216.0); }

struct Sink {
    std::vector<float>* px;
    std::vector<float>* py;
    std::vector<float>* vx;
    std::vector<float>* vy;
    uint64_t count = 0;
    void add(float x, float y, float u, float v) {
        if (px) { px->push_back(x); py->push_back(y); vx->push_back(u); vy->push_back(v); }
        count++;
    }
};

double value_noise(double x, double y, uint32_t key) {
    double fx = std::floor(x), fy = std::floor(y);
    int32_t ix = int32_t(fx), iy = int32_t(fy);
    double tx = x - fx, ty = y - fy;
    double sx = tx * tx * (3.0 - 2.0 * tx), sy = ty * ty * (3.0 - 2.0 * ty);
    auto lat = [&](int32_t i, int32_t j) {
        uint32_t h = uint32_t(i) * 73856093u ^ uint32_t(j) * 19349663u;
        return u01(key, h);
    };
    double a = lat(ix, iy), b = lat(ix + 1, iy), c = lat(ix, iy + 1), d = lat(ix + 1, iy + 1);
    double ab = a + (b - a) * sx, cd = c + (d - c) * sx;
    return ab + (cd - ab) * sy;
}

int generate(const apic_scene_params* p, Sink& out) {
    if (!p || p->width == 0 || p->height == 0) return APIC_ERR_INVALID_ARG;
    const uint32_t W = p->width, H = p->height;
    const float cs = p->cell_size > 0.0f ? p->cell_size : 1.0f / float(W > H ? W : H);
    if (p->kind == APIC_SCENE_REFERENCE_DEFAULT) {
        for (uint32_t y = 0; y < H; ++y)
            for (uint32_t x = 0; x < W; ++x) {
                bool border = x == 0 || x == W - 1 || y == 0 || y == H - 1;
                if (!border && x > 4 && x < W - 4 && y > 4 && y < H / 2)
                    for (int sy = 0; sy < 3; ++sy)
                        for (int sx = 0; sx < 3; ++sx)
                            out.add((float(x) + (float(sx) + 0.5f) / 3.0f) * cs,
                                    (float(y) + (float(sy) + 0.5f) / 3.0f) * cs, 0.0f, 0.0f);
            }
        return APIC_OK;
    }
    if (p->kind != APIC_SCENE_DAM_BREAK && p->kind != APIC_SCENE_DAM_BREAK_DISK && p->kind != APIC_SCENE_NOISE)
        return APIC_ERR_INVALID_ARG;
    const uint32_t sub = p->sub ? p->sub : 2;
    const uint32_t kx = stream_key(p->seed, 0), ky = stream_key(p->seed, 1);
    const uint32_t kg1 = stream_key(p->seed, 2), kg2 = stream_key(p->seed, 3);
    const uint32_t kn = stream_key(p->seed, 7);
    uint32_t id = 0;
    for (uint32_t j = 1; j + 1 < H; ++j)
        for (uint32_t i = 1; i + 1 < W; ++i) {
            double cx = (double(i) + 0.5) * cs, cy = (double(j) + 0.5) * cs;
            bool dam = false, disk = false;
            if (p->kind == APIC_SCENE_NOISE) {
                double period = p->noise_period > 0.0f ? p->noise_period : 0.05;
                dam = value_noise(cx / period, cy / period, kn) > double(p->noise_threshold);
            } else {
                dam = cx < double(p->fluid_x) && cy < double(p->fluid_y);
                if (!dam && p->kind == APIC_SCENE_DAM_BREAK_DISK) {
                    double dx = cx - double(p->disk_x), dy = cy - double(p->disk_y);
                    disk = dx * dx + dy * dy < double(p->disk_r) * double(p->disk_r);
                }
            }
            if (!dam && !disk) continue;
            for (uint32_t sy = 0; sy < sub; ++sy)
                for (uint32_t sx = 0; sx < sub; ++sx, ++id) {
                    double jx = u01(kx, id), jy = u01(ky, id);
                    float x = float((double(i) + (double(sx) + jx) / double(sub)) * cs);
                    float y = float((double(j) + (double(sy) + jy) / double(sub)) * cs);
                    float u = 0.0f, v = 0.0f;
                    if (disk) { u = p->disk_vx; v = p->disk_vy; }
                    if (p->kind == APIC_SCENE_NOISE) {
                        double a = u01(kg1, id), b = u01(kg2, id);
                        double r = std::sqrt(-2.0 * std::log(a > 1e-12 ? a : 1e-12));
                        double t = 6.283185307179586 * b;
                        u = float(double(p->vel_sigma) * r * std::cos(t));
                        v = float(double(p->vel_sigma) * r * std::sin(t));
                    }
                    out.add(x, y, u, v);
                }
        }
    return APIC_OK;
}

}  // namespace

extern "C" {

int apic_scene_count(const apic_scene_params* p, uint64_t* n_out) {
    if (!n_out) return APIC_ERR_INVALID_ARG;
    Sink s{nullptr, nullptr, nullptr, nullptr};
    int rc = generate(p, s);
    *n_out = s.count;
    return rc;
}

int apic_scene_fill(const apic_scene_params* p, uint64_t n, float* pos_x, float* pos_y, float* vel_x, float* vel_y) {
    if (!pos_x || !pos_y || !vel_x || !vel_y) return APIC_ERR_INVALID_ARG;
    std::vector<float> a, b, c, d;
    Sink s{&a, &b, &c, &d};
    int rc = generate(p, s);
    if (rc != APIC_OK) return rc;
    if (s.count != n) return APIC_ERR_INVALID_ARG;
    for (uint64_t i = 0; i < n; ++i) { pos_x[i] = a[i]; pos_y[i] = b[i]; vel_x[i] = c[i]; vel_y[i] = d[i]; }
    return APIC_OK;
}

}  // extern "C"
