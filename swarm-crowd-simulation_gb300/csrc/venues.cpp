// Synthetic venues and spawns: the inputs of the step, built once on the host.
//
// A hall is a rectangle of walls with door gaps. Its fields:
//   wall SDF   the exact horizontal signed distance to the union of the wall boxes (a box's 2D SDF, the minimum over
//              boxes), on a grid of wall_h;
//   nav field  the geodesic distance through the free nodes to the free nodes beyond the exit line, by the first-order
//              fast marching method (Sethian 1996) on a grid of nav_h; wall nodes get the largest free distance + 10 m,
//              so the normalised negative gradient never points into a wall.
// The lattice spawn draws from splitmix64 (Steele, Lea, Flood 2014) with Box-Muller normals, in double.

#include "../../include/swarm_cuda.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <queue>
#include <utility>
#include <vector>

namespace {

struct Box { double x0, y0, x1, y1; };

double sdBox(double px, double py, const Box& b) {
    const double cx = 0.5 * (b.x0 + b.x1), cy = 0.5 * (b.y0 + b.y1), hx = 0.5 * (b.x1 - b.x0), hy = 0.5 * (b.y1 - b.y0);
    const double qx = std::fabs(px - cx) - hx, qy = std::fabs(py - cy) - hy;
    const double ox = std::max(qx, 0.0), oy = std::max(qy, 0.0);
    return std::sqrt(ox * ox + oy * oy) + std::min(std::max(qx, qy), 0.0);
}

bool validSpec(const SwarmHallSpec* s) {
    if (!s || !(s->size_x > 0) || !(s->size_y > 0) || !(s->wall_thickness > 0) || !(s->exit_depth >= 0) || !(s->margin >= 0) ||
        !(s->wall_h > 0) || !(s->nav_h > 0) || !(s->cell > 0) || s->n_doors < 0 || s->n_doors > 8)
        return false;
    for (int d = 0; d < s->n_doors; ++d)
        if (s->door_wall[d] < 0 || s->door_wall[d] > 3 || !(s->door_width[d] > 0)) return false;
    return true;
}

// The wall boxes: each wall as the intervals along it that no door cuts
std::vector<Box> wallBoxes(const SwarmHallSpec* s) {
    const double hx = 0.5 * s->size_x, hy = 0.5 * s->size_y, t = s->wall_thickness;
    std::vector<Box> boxes;
    for (int w = 0; w < 4; ++w) {
        // the wall's extent along its own axis, and its span across
        const bool alongY = w < 2;                       // the x walls run along y
        const double lo = alongY ? -hy - t : -hx, hi = alongY ? hy + t : hx;
        std::vector<std::pair<double, double>> cuts;
        for (int d = 0; d < s->n_doors; ++d)
            if (s->door_wall[d] == w) cuts.push_back({s->door_center[d] - 0.5 * s->door_width[d], s->door_center[d] + 0.5 * s->door_width[d]});
        std::sort(cuts.begin(), cuts.end());
        double a = lo;
        auto emit = [&](double u0, double u1) {
            if (u1 <= u0) return;
            if (w == 0) boxes.push_back({-hx - t, u0, -hx, u1});
            if (w == 1) boxes.push_back({hx, u0, hx + t, u1});
            if (w == 2) boxes.push_back({u0, -hy - t, u1, -hy});
            if (w == 3) boxes.push_back({u0, hy, u1, hy + t});
        };
        for (auto& c : cuts) { emit(a, std::max(a, c.first)); a = std::max(a, c.second); }
        emit(a, hi);
    }
    return boxes;
}

double wallSdf(const std::vector<Box>& boxes, double x, double y) {
    double d = 1e9;
    for (const Box& b : boxes) d = std::min(d, sdBox(x, y, b));
    return d;
}

uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
double uniform01(uint64_t& s) { return double(splitmix64(s) >> 11) * 0x1.0p-53; }   // [0, 1)

}  // namespace

extern "C" int swarm_hall_layout(const SwarmHallSpec* s, SwarmVenue* v) {
    if (!validSpec(s) || !v) return SWARM_E_INVALID;
    *v = SwarmVenue{};
    const double hx = 0.5 * s->size_x, hy = 0.5 * s->size_y, t = s->wall_thickness;
    const double ex = hx + t + s->exit_depth, ey = hy + t + s->exit_depth;
    const double dx = ex + s->margin, dy = ey + s->margin;
    v->kind = SWARM_VENUE_GRID;
    v->grid_res_x = int(std::ceil(2.0 * dx / s->cell));
    v->grid_res_y = int(std::ceil(2.0 * dy / s->cell));
    v->domain_span_x = float(v->grid_res_x * double(s->cell));
    v->domain_span_y = float(v->grid_res_y * double(s->cell));
    v->domain_min_x = -0.5f * v->domain_span_x;
    v->domain_min_y = -0.5f * v->domain_span_y;
    v->exit_lo_x = float(-ex); v->exit_hi_x = float(ex);
    v->exit_lo_y = float(-ey); v->exit_hi_y = float(ey);
    v->exit_max_z = 1e30f;   // a flat hall: the exit line counts at any height
    v->wall_h = s->wall_h;
    v->wall_origin_x = v->domain_min_x; v->wall_origin_y = v->domain_min_y;
    v->wall_nx = int(std::lround(double(v->domain_span_x) / s->wall_h)) + 1;
    v->wall_ny = int(std::lround(double(v->domain_span_y) / s->wall_h)) + 1;
    v->nav_h = s->nav_h;
    v->nav_origin_x = v->domain_min_x; v->nav_origin_y = v->domain_min_y;
    v->nav_nx = int(std::lround(double(v->domain_span_x) / s->nav_h)) + 1;
    v->nav_ny = int(std::lround(double(v->domain_span_y) / s->nav_h)) + 1;
    v->n_exits = s->n_doors;
    v->metric_res = int(std::ceil(std::max(v->domain_span_x, v->domain_span_y) / 16.0)) * 16;   // 1 m cells, a multiple of 16
    v->metric_center_x = 0.0f; v->metric_center_y = 0.0f;
    return SWARM_OK;
}

extern "C" int swarm_hall_fields(const SwarmHallSpec* s, const SwarmVenue* v, float* wall, float* nav, float* exitBoxes) {
    if (!validSpec(s) || !v || !wall || !nav) return SWARM_E_INVALID;
    const std::vector<Box> boxes = wallBoxes(s);
    const double hx = 0.5 * s->size_x, hy = 0.5 * s->size_y, t = s->wall_thickness;
    // wall SDF
    for (int j = 0; j < v->wall_ny; ++j)
        for (int i = 0; i < v->wall_nx; ++i)
            wall[size_t(j) * size_t(v->wall_nx) + size_t(i)] =
                float(wallSdf(boxes, double(v->wall_origin_x) + i * double(v->wall_h), double(v->wall_origin_y) + j * double(v->wall_h)));
    // fast marching on the nav grid
    const int nx = v->nav_nx, ny = v->nav_ny;
    const size_t M = size_t(nx) * size_t(ny);
    const double h = v->nav_h, INF = std::numeric_limits<double>::infinity();
    std::vector<double> D(M, INF);
    std::vector<uint8_t> state(M, 0);   // 0 far, 1 trial, 2 known, 3 wall
    using Item = std::pair<double, size_t>;
    std::priority_queue<Item, std::vector<Item>, std::greater<Item>> heap;
    for (int j = 0; j < ny; ++j) {
        for (int i = 0; i < nx; ++i) {
            const size_t k = size_t(j) * size_t(nx) + size_t(i);
            const double x = double(v->nav_origin_x) + i * h, y = double(v->nav_origin_y) + j * h;
            if (wallSdf(boxes, x, y) <= 0.0) { state[k] = 3; continue; }
            if (x < v->exit_lo_x || x > v->exit_hi_x || y < v->exit_lo_y || y > v->exit_hi_y) { D[k] = 0.0; state[k] = 1; heap.push({0.0, k}); }
        }
    }
    auto val = [&](int i, int j) -> double {
        if (i < 0 || j < 0 || i >= nx || j >= ny) return INF;
        const size_t k = size_t(j) * size_t(nx) + size_t(i);
        return state[k] == 2 ? D[k] : INF;
    };
    while (!heap.empty()) {
        const auto [d, k] = heap.top();
        heap.pop();
        if (state[k] == 2 || d > D[k]) continue;
        state[k] = 2;
        const int i = int(k % size_t(nx)), j = int(k / size_t(nx));
        const int ni[4] = {i - 1, i + 1, i, i}, nj[4] = {j, j, j - 1, j + 1};
        for (int q = 0; q < 4; ++q) {
            if (ni[q] < 0 || nj[q] < 0 || ni[q] >= nx || nj[q] >= ny) continue;
            const size_t kk = size_t(nj[q]) * size_t(nx) + size_t(ni[q]);
            if (state[kk] >= 2) continue;
            const double a = std::min(val(ni[q] - 1, nj[q]), val(ni[q] + 1, nj[q]));
            const double b = std::min(val(ni[q], nj[q] - 1), val(ni[q], nj[q] + 1));
            double T;
            if (std::isinf(a) || std::isinf(b) || std::fabs(a - b) >= h) T = std::min(a, b) + h;
            else T = 0.5 * (a + b + std::sqrt(2.0 * h * h - (a - b) * (a - b)));
            if (T < D[kk]) { D[kk] = T; state[kk] = 1; heap.push({T, kk}); }
        }
    }
    double maxFree = 0.0;
    for (size_t k = 0; k < M; ++k) if (state[k] == 2) maxFree = std::max(maxFree, D[k]);
    for (size_t k = 0; k < M; ++k) nav[k] = float(state[k] == 2 ? D[k] : maxFree + 10.0);
    // exit boxes: each door's opening, from the interior face out to the domain edge
    if (exitBoxes) {
        for (int d = 0; d < s->n_doors; ++d) {
            const double c0 = s->door_center[d] - 0.5 * s->door_width[d], c1 = s->door_center[d] + 0.5 * s->door_width[d];
            const double fx = -double(v->domain_min_x), fy = -double(v->domain_min_y);
            double b[4];
            switch (s->door_wall[d]) {
                case 0: b[0] = -fx; b[1] = c0; b[2] = -hx; b[3] = c1; break;
                case 1: b[0] = hx; b[1] = c0; b[2] = fx; b[3] = c1; break;
                case 2: b[0] = c0; b[1] = -fy; b[2] = c1; b[3] = -hy; break;
                default: b[0] = c0; b[1] = hy; b[2] = c1; b[3] = fy; break;
            }
            for (int q = 0; q < 4; ++q) exitBoxes[4 * d + q] = float(b[q]);
        }
    }
    (void)t;
    return SWARM_OK;
}

extern "C" int swarm_spawn_lattice(int nx, int ny, int n, float spacing, float cx, float cy, float jitter, uint64_t seed,
                                   float r_lo, float r_hi, float v_mean, float v_sd, float v_lo, float v_hi,
                                   float* boids, float* radius, float* v0) {
    if (nx <= 0 || ny <= 0 || n <= 0 || n > nx * ny || !boids || !radius || !v0) return SWARM_E_INVALID;
    uint64_t s = seed;
    const double pi2 = 6.283185307179586;
    for (int i = 0; i < n; ++i) {
        const int c = i % nx, r = i / nx;
        const double jx = (2.0 * uniform01(s) - 1.0) * jitter, jy = (2.0 * uniform01(s) - 1.0) * jitter;
        const double rad = r_lo + (r_hi - r_lo) * uniform01(s);
        const double u1 = 1.0 - uniform01(s), u2 = uniform01(s);
        const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(pi2 * u2);
        const double v = std::min(std::max(v_mean + v_sd * z, double(v_lo)), double(v_hi));
        float* b = boids + size_t(i) * 8;
        b[0] = float(cx + (c - 0.5 * (nx - 1)) * spacing + jx);
        b[1] = float(cy + (r - 0.5 * (ny - 1)) * spacing + jy);
        b[2] = float(rad);
        b[3] = 1.0f;
        b[4] = b[5] = b[6] = b[7] = 0.0f;
        radius[i] = float(rad);
        v0[i] = float(v);
    }
    return SWARM_OK;
}

extern "C" int swarm_metric_thresholds_grid(const SwarmVenue* v, int res, uint32_t* out) {
    if (!v || !out || res <= 0 || !v->wall_sdf || v->wall_nx < 2 || v->wall_ny < 2 || !(v->wall_h > 0)) return SWARM_E_INVALID;
    // persons per m^2: Fruin's LoS E and LoS F, and the crush level (the reference's metrics.hpp thresholds)
    const double thresholds[3] = {1.08, 2.17, 5.0};
    const int sub = 40;
    const double inv = 1.0 / v->wall_h;
    auto wallAt = [&](double x, double y) {
        double fx = (x - v->wall_origin_x) * inv, fy = (y - v->wall_origin_y) * inv;
        if (fx < 0 || fy < 0 || fx > v->wall_nx - 1 || fy > v->wall_ny - 1) return 1.0;
        int ix = std::min(int(fx), v->wall_nx - 2), iy = std::min(int(fy), v->wall_ny - 2);
        double wx = fx - ix, wy = fy - iy;
        const float* W = v->wall_sdf;
        size_t r0 = size_t(iy) * size_t(v->wall_nx) + size_t(ix), r1 = r0 + size_t(v->wall_nx);
        return (W[r0] * (1 - wx) + W[r0 + 1] * wx) * (1 - wy) + (W[r1] * (1 - wx) + W[r1 + 1] * wx) * wy;
    };
    for (int iy = 0; iy < res; ++iy) {
        for (int ix = 0; ix < res; ++ix) {
            int free = 0;
            for (int sy = 0; sy < sub; ++sy) {
                for (int sx = 0; sx < sub; ++sx) {
                    const double x = v->metric_center_x + (ix - 0.5 * res) + (sx + 0.5) / sub;
                    const double y = v->metric_center_y + (iy - 0.5 * res) + (sy + 0.5) / sub;
                    if (x < v->exit_lo_x || x > v->exit_hi_x || y < v->exit_lo_y || y > v->exit_hi_y) continue;
                    free += wallAt(x, y) > 0.0;
                }
            }
            const double area = double(free) / double(sub * sub);
            uint32_t* t = out + 4 * (size_t(iy) * size_t(res) + size_t(ix));
            for (int k = 0; k < 3; ++k) {
                const double m = std::ceil(thresholds[k] * area * 65536.0);
                t[k] = area < 0.1 ? 0xFFFFFFFFu : uint32_t(std::min(std::max(m, 1.0), 4294967295.0));
            }
            t[3] = 0xFFFFFFFFu;
        }
    }
    return SWARM_OK;
}
