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
#include <atomic>
#include <cmath>
#include <cstdint>
#include <limits>
#include <queue>
#include <thread>
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

// First-order fast marching (Sethian 1996) on an nx x ny grid of spacing h. kind per node: 0 free, 1 source (0),
// 3 wall (never entered). The local step is h / speed (speed: per node, null = 1): the travel distance in
// flat-floor metres. Nodes never reached and walls get the largest reached value + 10 m, so the normalised negative
// gradient never points into a wall.
void fastMarchCpu(int nx, int ny, double h, std::vector<uint8_t> state, const float* speed, float* out) {
    const size_t M = size_t(nx) * size_t(ny);
    const double INF = std::numeric_limits<double>::infinity();
    std::vector<double> D(M, INF);
    using Item = std::pair<double, size_t>;
    std::priority_queue<Item, std::vector<Item>, std::greater<Item>> heap;
    for (size_t k = 0; k < M; ++k) {   // state: 0 far, 1 trial, 2 known, 3 wall
        if (state[k] == 1) { D[k] = 0.0; heap.push({0.0, k}); }
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
            const double hs = speed ? h / double(speed[kk]) : h;
            const double a = std::min(val(ni[q] - 1, nj[q]), val(ni[q] + 1, nj[q]));
            const double b = std::min(val(ni[q], nj[q] - 1), val(ni[q], nj[q] + 1));
            double T;
            if (std::isinf(a) || std::isinf(b) || std::fabs(a - b) >= hs) T = std::min(a, b) + hs;
            else T = 0.5 * (a + b + std::sqrt(2.0 * hs * hs - (a - b) * (a - b)));
            if (T < D[kk]) { D[kk] = T; state[kk] = 1; heap.push({T, kk}); }
        }
    }
    double maxFree = 0.0;
    for (size_t k = 0; k < M; ++k) if (state[k] == 2) maxFree = std::max(maxFree, D[k]);
    for (size_t k = 0; k < M; ++k) out[k] = float(state[k] == 2 ? D[k] : maxFree + 10.0);
}

// Runs f(j) for j in [0, n) over the host's threads
template <class F>
void parallelRows(int n, F f) {
    const int t = std::max(1, std::min(int(std::thread::hardware_concurrency()), 32));
    std::vector<std::thread> pool;
    for (int i = 0; i < t; ++i)
        pool.emplace_back([&, i] { for (int j = i; j < n; j += t) f(j); });
    for (auto& th : pool) th.join();
}

// The blocked band of a nav field: the wall nodes (kind 3: the walls and the clearance around them) within maxDist of a
// node the solver reached get the value of the nearest reached node (Euclidean, over node centres) plus k x that
// distance, instead of the solver's plain fill (largest reached value + 10 m). Beside a
// wall's clearance band the field then rises gently into the band: its normalised negative gradient keeps the
// route's direction with a push away from the wall, where the cliff of the plain fill turned it straight away from
// the wall (which held pairs of agents face to face at the ends of thin walls). Wall nodes farther from every reached
// node, and free nodes no exit reaches, keep the plain fill. The nearest reached node comes from an exact separable distance transform with the
// nearest feature tracked (the lower envelope of parabolas, Felzenszwalb and Huttenlocher, Theory of Computing 8,
// 2012): each column's nearest reached row, then along each row the least (x - x')^2 + (row distance at x')^2,
// the first (lowest x', then lowest row) on a tie.
void fillBand(int nx, int ny, double h, float* out, double k, double maxDist, const uint8_t* kind) {
    const size_t m = size_t(nx) * size_t(ny);
    // the plain fill: the largest value, 10 m above every reached one (none when every node was reached)
    float top = -std::numeric_limits<float>::infinity(), second = top;
    for (size_t q = 0; q < m; ++q) top = std::max(top, out[q]);
    for (size_t q = 0; q < m; ++q) if (out[q] < top) second = std::max(second, out[q]);
    if (!(double(top) - double(second) >= 9.0)) return;
    auto reached = [&](size_t q) { return out[q] < top; };
    const int64_t INF = std::numeric_limits<int64_t>::max() / 4;
    // column pass: squared row distance to the nearest reached node of the column, and its row
    std::vector<int64_t> col(m, INF);
    std::vector<int32_t> colRow(m, -1);
    parallelRows(nx, [&](int i) {
        int last = -1;
        for (int j = 0; j < ny; ++j) {
            const size_t q = size_t(j) * size_t(nx) + size_t(i);
            if (reached(q)) last = j;
            if (last >= 0) { col[q] = int64_t(j - last) * int64_t(j - last); colRow[q] = last; }
        }
        int next = -1;
        for (int j = ny - 1; j >= 0; --j) {
            const size_t q = size_t(j) * size_t(nx) + size_t(i);
            if (reached(q)) next = j;
            if (next >= 0) {
                const int64_t d = int64_t(next - j) * int64_t(next - j);
                if (d < col[q]) { col[q] = d; colRow[q] = next; }
            }
        }
    });
    // row pass: the lower envelope of the parabolas (x - x')^2 + col(x') over the columns with a reached node
    std::vector<float> filled(out, out + m);
    parallelRows(ny, [&](int j) {
        const size_t base = size_t(j) * size_t(nx);
        std::vector<int> v(static_cast<size_t>(nx));
        std::vector<double> z(size_t(nx) + 1);
        int kk = -1;
        for (int q = 0; q < nx; ++q) {
            const int64_t fq = col[base + size_t(q)];
            if (fq >= INF) continue;
            while (kk >= 0) {
                const int p = v[size_t(kk)];
                const double sx = (double(fq + int64_t(q) * q) - double(col[base + size_t(p)] + int64_t(p) * p)) / (2.0 * (q - p));
                if (sx <= z[size_t(kk)]) { --kk; continue; }
                ++kk;
                v[size_t(kk)] = q;
                z[size_t(kk)] = sx;
                z[size_t(kk) + 1] = std::numeric_limits<double>::infinity();
                break;
            }
            if (kk < 0) {
                kk = 0;
                v[0] = q;
                z[0] = -std::numeric_limits<double>::infinity();
                z[1] = std::numeric_limits<double>::infinity();
            }
        }
        if (kk < 0) return;   // no reached node in any column
        int e = 0;
        for (int x = 0; x < nx; ++x) {
            const size_t q = base + size_t(x);
            while (z[size_t(e) + 1] < double(x)) ++e;
            if (reached(q) || kind[q] != 3) continue;
            const int fx = v[size_t(e)];
            const int64_t d2 = int64_t(x - fx) * int64_t(x - fx) + col[base + size_t(fx)];
            const double dist = std::sqrt(double(d2)) * h;
            if (dist > maxDist) continue;
            const size_t src = size_t(colRow[base + size_t(fx)]) * size_t(nx) + size_t(fx);
            filled[q] = float(double(out[src]) + k * dist);
        }
    });
    std::copy(filled.begin(), filled.end(), out);
}

// The bowl's band fill: 3 m of field per metre into the band, up to 1 m from the reached nodes. Measured on the
// 63 488-seat bowl (GB300, bit-exact step): slopes 1.5, 3 and 6 empty it within 10 000 steps, the plain fill left 4
// agents after 24 000 steps and a slope of 12 left 2.
constexpr double BAND_SLOPE = 3.0, BAND_REACH = 1.0;

std::atomic<int> navSolver{SWARM_NAV_CPU};

// The builders' solver: fast marching here, or the GPU solver (the same floats) when selected
// (SWARM_HOST_ONLY: this file compiled alone, without the CUDA library, for a host process that only builds venues;
// there the GPU solver cannot be selected.)
int fastMarch(int nx, int ny, double h, std::vector<uint8_t> state, const float* speed, float* out) {
#ifndef SWARM_HOST_ONLY
    if (navSolver.load() == SWARM_NAV_GPU) return swarm_nav_field_gpu(nx, ny, h, state.data(), speed, out, nullptr);
#endif
    fastMarchCpu(nx, ny, h, std::move(state), speed, out);
    return SWARM_OK;
}

}  // namespace

extern "C" int swarm_set_nav_solver(int solver) {
    if (solver != SWARM_NAV_CPU && solver != SWARM_NAV_GPU) return SWARM_E_INVALID;
#ifdef SWARM_HOST_ONLY
    if (solver == SWARM_NAV_GPU) return SWARM_E_INVALID;
#endif
    return navSolver.exchange(solver);
}

extern "C" int swarm_nav_field_cpu(int nx, int ny, double h, const uint8_t* kind, const float* speed, float* out) {
    if (nx < 2 || ny < 2 || !(h > 0.0) || !kind || !out) return SWARM_E_INVALID;
    const size_t m = size_t(nx) * size_t(ny);
    if (speed)
        for (size_t k = 0; k < m; ++k)
            if (kind[k] == 0 && !(speed[k] > 0.0f)) return SWARM_E_INVALID;
    fastMarchCpu(nx, ny, h, std::vector<uint8_t>(kind, kind + m), speed, out);
    return SWARM_OK;
}

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

namespace {

// The hall's nav node kinds: sources beyond the exit line, walls where the wall SDF is <= 0
std::vector<uint8_t> hallNavKind(const SwarmVenue* v, const std::vector<Box>& boxes) {
    const int nx = v->nav_nx, ny = v->nav_ny;
    std::vector<uint8_t> kind(size_t(nx) * size_t(ny), 0);
    for (int j = 0; j < ny; ++j) {
        for (int i = 0; i < nx; ++i) {
            const size_t k = size_t(j) * size_t(nx) + size_t(i);
            const double x = double(v->nav_origin_x) + i * double(v->nav_h), y = double(v->nav_origin_y) + j * double(v->nav_h);
            if (wallSdf(boxes, x, y) <= 0.0) kind[k] = 3;
            else if (x < v->exit_lo_x || x > v->exit_hi_x || y < v->exit_lo_y || y > v->exit_hi_y) kind[k] = 1;
        }
    }
    return kind;
}

// Each door's opening, from the interior face out to the domain edge (lo_x, lo_y, hi_x, hi_y)
void hallExitBoxes(const SwarmHallSpec* s, const SwarmVenue* v, float* exitBoxes) {
    const double hx = 0.5 * s->size_x, hy = 0.5 * s->size_y;
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

// Each exit's own distance field: the venue's nav kinds with only exit e's sources (every source node belongs to the
// exit whose box lies nearest, the first on a tie; a box holds its own nodes at distance 0); the other exits'
// sources become walls, so no path leaves through one door and comes back in through another. `hallOutside`: source
// nodes outside every box are the outside of a hall, reached only through its doors: walls for every exit.
int exitFields(const SwarmVenue* v, const std::vector<uint8_t>& kind, const float* speed, const float* boxes, int nExits,
               float* fields, bool hallOutside, double bandSlope = 0.0) {
    const int nx = v->nav_nx, ny = v->nav_ny;
    const size_t m = size_t(nx) * size_t(ny);
    std::vector<int8_t> owner(m, -1);
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const size_t k = size_t(j) * size_t(nx) + size_t(i);
            if (kind[k] != 1) continue;
            const double x = double(v->nav_origin_x) + i * double(v->nav_h), y = double(v->nav_origin_y) + j * double(v->nav_h);
            double best = 0.0;
            for (int e = 0; e < nExits; ++e) {
                const double dx = std::max({double(boxes[4 * e]) - x, 0.0, x - double(boxes[4 * e + 2])});
                const double dy = std::max({double(boxes[4 * e + 1]) - y, 0.0, y - double(boxes[4 * e + 3])});
                const double d = dx * dx + dy * dy;
                if (hallOutside && d > 0.0) continue;
                if (owner[k] < 0 || d < best) { owner[k] = int8_t(e); best = d; }
            }
        }
    for (int e = 0; e < nExits; ++e) {
        std::vector<uint8_t> ke(kind);
        for (size_t k = 0; k < m; ++k)
            if (ke[k] == 1 && owner[k] != e) ke[k] = 3;
        if (const int rc = fastMarch(nx, ny, v->nav_h, std::move(ke), speed, fields + size_t(e) * m); rc != SWARM_OK) return rc;
        if (bandSlope > 0.0) fillBand(nx, ny, v->nav_h, fields + size_t(e) * m, bandSlope, BAND_REACH, kind.data());
    }
    return SWARM_OK;
}

}  // namespace

extern "C" int swarm_hall_fields(const SwarmHallSpec* s, const SwarmVenue* v, float* wall, float* nav, float* exitBoxes) {
    if (!validSpec(s) || !v || !wall || !nav) return SWARM_E_INVALID;
    const std::vector<Box> boxes = wallBoxes(s);
    // wall SDF
    for (int j = 0; j < v->wall_ny; ++j)
        for (int i = 0; i < v->wall_nx; ++i)
            wall[size_t(j) * size_t(v->wall_nx) + size_t(i)] =
                float(wallSdf(boxes, double(v->wall_origin_x) + i * double(v->wall_h), double(v->wall_origin_y) + j * double(v->wall_h)));
    // fast marching on the nav grid
    if (const int rc = fastMarch(v->nav_nx, v->nav_ny, v->nav_h, hallNavKind(v, boxes), nullptr, nav); rc != SWARM_OK) return rc;
    if (exitBoxes) hallExitBoxes(s, v, exitBoxes);
    return SWARM_OK;
}

extern "C" int swarm_hall_exit_fields(const SwarmHallSpec* s, const SwarmVenue* v, float* fields, float* width, uint8_t* type) {
    if (!validSpec(s) || !v || !fields || s->n_doors < 1 || s->n_doors > SWARM_CHOICE_MAX_EXITS) return SWARM_E_INVALID;
    std::vector<float> boxes(size_t(4) * size_t(s->n_doors));
    hallExitBoxes(s, v, boxes.data());
    for (int d = 0; d < s->n_doors; ++d) {
        if (width) width[d] = s->door_width[d];
        if (type) type[d] = 1;
    }
    // the per-exit fields see the hall's interior and its door openings only: every node outside the interior and
    // outside the door boxes is a wall (the outside is reached through the doors alone)
    std::vector<uint8_t> kind = hallNavKind(v, wallBoxes(s));
    const double hx = 0.5 * s->size_x, hy = 0.5 * s->size_y;
    for (int j = 0; j < v->nav_ny; ++j)
        for (int i = 0; i < v->nav_nx; ++i) {
            const double x = double(v->nav_origin_x) + i * double(v->nav_h), y = double(v->nav_origin_y) + j * double(v->nav_h);
            if (std::fabs(x) <= hx && std::fabs(y) <= hy) continue;
            bool door = false;
            for (int d = 0; d < s->n_doors && !door; ++d)
                door = x >= boxes[size_t(4 * d)] && x <= boxes[size_t(4 * d + 2)] && y >= boxes[size_t(4 * d + 1)] && y <= boxes[size_t(4 * d + 3)];
            if (!door) kind[size_t(j) * size_t(v->nav_nx) + size_t(i)] = 3;
        }
    return exitFields(v, kind, nullptr, boxes.data(), s->n_doors, fields, true);
}

// ---- the seated bowl ----
namespace {

bool validBowl(const SwarmBowlSpec* s) {
    return s && s->sectors >= 3 && s->rows >= 1 && s->seats >= 1 && s->seat_width > 0 && s->row_pitch > 0 && s->rise >= 0 &&
           s->gangway > 0 && s->vomitory_width > 0 && s->vomitory_row >= 0 && s->vomitory_row < s->rows &&
           s->perimeter_exits >= 0 && s->perimeter_exits <= s->sectors && s->perimeter_exit_width > 0 && s->concourse > 0 &&
           s->aisle >= 0 && s->clearance >= 0 &&
           s->stair_speed > 0 && s->wall_h > 0 && s->nav_h > 0 && s->cell > 0 && s->sectors + s->perimeter_exits <= 56;
}

// The bowl in each sector's frame: u along its rows, w outward from the pitch wall (the polygon's inner edge)
struct Bowl {
    const SwarmBowlSpec& s;
    double dphi, halfRow, rin, depth, outerW;
    const double wallT = 0.3, rowWallT = 0.1;
    std::vector<double> c, sn;
    std::vector<uint8_t> exitSector;
    explicit Bowl(const SwarmBowlSpec& sp) : s(sp) {
        dphi = 2.0 * 3.141592653589793 / s.sectors;
        halfRow = 0.5 * s.seats * double(s.seat_width);
        rin = (2.0 * halfRow + s.gangway) / (2.0 * std::tan(0.5 * dphi));   // blocks gangway apart at the pitch wall
        depth = s.rows * double(s.row_pitch);
        outerW = depth + s.concourse;
        c.resize(size_t(s.sectors)); sn.resize(size_t(s.sectors)); exitSector.assign(size_t(s.sectors), 0);
        for (int k = 0; k < s.sectors; ++k) { c[size_t(k)] = std::cos(k * dphi); sn[size_t(k)] = std::sin(k * dphi); }
        for (int e = 0; e < s.perimeter_exits; ++e) exitSector[size_t((long(e) * s.sectors) / s.perimeter_exits)] = 1;
    }
    double outerRadius() const { return (rin + outerW + wallT) / std::cos(0.5 * dphi); }
    int sector(double x, double y) const {
        int k = int(std::lround(std::atan2(y, x) / dphi)) % s.sectors;
        return k < 0 ? k + s.sectors : k;
    }
    void local(int k, double x, double y, double& u, double& w) const {
        k = ((k % s.sectors) + s.sectors) % s.sectors;
        w = x * c[size_t(k)] + y * sn[size_t(k)] - rin;
        u = -x * sn[size_t(k)] + y * c[size_t(k)];
    }
    static double box(double u, double w, double u0, double u1, double w0, double w1) {
        return sdBox(u, w, Box{u0, w0, u1, w1});
    }
    // the walls of sector k near (u, w): the pitch wall (beyond the cross-aisle), the nearest row edges (the back edge
    // of every row), the outer wall (with its exit gap)
    double sectorSdf(int k, double u, double w) const {
        const double half = std::tan(0.5 * dphi), a = s.aisle;
        const double lf = (rin - a) * half + wallT, lo = (rin + outerW + wallT) * half + wallT;
        double d = box(u, w, -lf, lf, -a - wallT, -a);
        const int j0 = int(std::lround(w / s.row_pitch));
        for (int j = j0 - 1; j <= j0 + 1; ++j) {
            if (j < 1 || j > s.rows) continue;
            const double wj = j * double(s.row_pitch);
            d = std::min(d, box(u, w, -halfRow, halfRow, wj - 0.5 * rowWallT, wj + 0.5 * rowWallT));
        }
        const int kk = ((k % s.sectors) + s.sectors) % s.sectors;
        if (exitSector[size_t(kk)]) {
            const double g = 0.5 * s.perimeter_exit_width;
            d = std::min(d, box(u, w, -lo, -g, outerW, outerW + wallT));
            d = std::min(d, box(u, w, g, lo, outerW, outerW + wallT));
        } else {
            d = std::min(d, box(u, w, -lo, lo, outerW, outerW + wallT));
        }
        return d;
    }
    double sdf(double x, double y) const {
        const int k = sector(x, y);
        double d = 1e9;
        for (int q = k - 1; q <= k + 1; ++q) {
            double u, w;
            local(q, x, y, u, w);
            d = std::min(d, sectorSdf(q, u, w));
        }
        return d;
    }
    // floor height and speed factor: row treads, gangway stairs of half-rise steps, the concourse
    void floorAt(double x, double y, double& h, double& speed) const {
        double u, w;
        local(sector(x, y), x, y, u, w);
        speed = 1.0;
        if (w < 0.0) { h = 0.0; return; }
        if (w >= depth) { h = s.rows * double(s.rise); return; }
        if (std::fabs(u) <= halfRow) { h = std::floor(w / s.row_pitch) * s.rise; return; }
        h = std::floor(w / (0.5 * s.row_pitch)) * (0.5 * s.rise);
        speed = s.stair_speed;
    }
    // beyond an exit: a vomitory across a gangway at the vomitory row, or past a perimeter gap
    bool isExit(double x, double y) const {
        const int k = sector(x, y);
        double u, w;
        local(k, x, y, u, w);
        const double vw0 = s.vomitory_row * double(s.row_pitch);
        if (std::fabs(u) > halfRow && w >= vw0 && w < vw0 + s.row_pitch) {
            for (int side = -1; side <= 1; side += 2) {   // the bisectors with the neighbouring sectors
                const double b = (k + 0.5 * side) * dphi;
                if (std::fabs(-x * std::sin(b) + y * std::cos(b)) <= 0.5 * s.vomitory_width) return true;
            }
        }
        return exitSector[size_t(k)] && w >= outerW + wallT && std::fabs(u) < 0.5 * s.perimeter_exit_width;
    }
};

}  // namespace

extern "C" int swarm_bowl_layout(const SwarmBowlSpec* s, SwarmVenue* v) {
    if (!validBowl(s) || !v) return SWARM_E_INVALID;
    const Bowl B(*s);
    *v = SwarmVenue{};
    const double half = std::ceil((B.outerRadius() + 2.0) / s->cell) * s->cell;
    v->kind = SWARM_VENUE_GRID;
    v->grid_res_x = v->grid_res_y = int(std::lround(2.0 * half / s->cell));
    v->domain_span_x = v->domain_span_y = float(v->grid_res_x * double(s->cell));
    v->domain_min_x = v->domain_min_y = -0.5f * v->domain_span_x;
    v->exit_lo_x = v->exit_lo_y = v->domain_min_x;   // (the exit mask decides)
    v->exit_hi_x = v->exit_hi_y = -v->domain_min_x;
    v->exit_max_z = 1e30f;
    v->wall_h = s->wall_h;
    v->wall_origin_x = v->wall_origin_y = v->domain_min_x;
    v->wall_nx = v->wall_ny = int(std::lround(double(v->domain_span_x) / s->wall_h)) + 1;
    v->nav_h = s->nav_h;
    v->nav_origin_x = v->nav_origin_y = v->domain_min_x;
    v->nav_nx = v->nav_ny = int(std::lround(double(v->domain_span_x) / s->nav_h)) + 1;
    v->n_exits = s->sectors + s->perimeter_exits;
    v->metric_res = int(std::ceil(double(v->domain_span_x) / 16.0)) * 16;
    return SWARM_OK;
}

namespace {

// The bowl's nav node kinds (walls within the clearance, sources at the exits), speed factors and exit mask
void bowlNav(const SwarmBowlSpec* s, const SwarmVenue* v, const Bowl& B, std::vector<uint8_t>& kind, std::vector<float>& speed,
             uint8_t* mask) {
    const int nn = v->nav_nx;
    kind.assign(size_t(nn) * size_t(v->nav_ny), 0);
    speed.assign(kind.size(), 0.0f);
    parallelRows(v->nav_ny, [&](int j) {
        for (int i = 0; i < nn; ++i) {
            const double x = double(v->nav_origin_x) + i * double(v->nav_h), y = double(v->nav_origin_y) + j * double(v->nav_h);
            const size_t k = size_t(j) * size_t(nn) + size_t(i);
            double h, sp;
            B.floorAt(x, y, h, sp);
            speed[k] = float(sp);
            const bool ex = B.isExit(x, y);
            if (mask) mask[k] = ex ? 1 : 0;
            // blocked within the clearance of a wall (the largest body radius): a thin row wall between nodes still
            // cuts the field, and the paths round every wall end at a distance a body can keep, so e_goal never
            // points into the wall an agent touches
            kind[k] = B.sdf(x, y) <= double(s->clearance) ? 3 : (ex ? 1 : 0);
        }
    });
}

// Each exit's bounding box (lo_x, lo_y, hi_x, hi_y): the sectors' vomitories, then the perimeter exits
void bowlExitBoxes(const SwarmBowlSpec* s, const Bowl& B, float* exitBoxes) {
    auto bound = [&](int e, int k, double u0, double u1, double w0, double w1) {
        double lo[2] = {1e30, 1e30}, hi[2] = {-1e30, -1e30};
        for (int q = 0; q < 4; ++q) {
            const double u = (q & 1) ? u1 : u0, w = (q & 2) ? w1 : w0;
            const double x = (B.rin + w) * B.c[size_t(k)] - u * B.sn[size_t(k)], y = (B.rin + w) * B.sn[size_t(k)] + u * B.c[size_t(k)];
            lo[0] = std::min(lo[0], x); lo[1] = std::min(lo[1], y); hi[0] = std::max(hi[0], x); hi[1] = std::max(hi[1], y);
        }
        exitBoxes[4 * e] = float(lo[0]); exitBoxes[4 * e + 1] = float(lo[1]);
        exitBoxes[4 * e + 2] = float(hi[0]); exitBoxes[4 * e + 3] = float(hi[1]);
    };
    const double vw0 = s->vomitory_row * double(s->row_pitch);
    for (int k = 0; k < s->sectors; ++k) {   // the vomitory between sector k and k + 1, in the bisector's frame
        const double b = (k + 0.5) * B.dphi, cb = std::cos(b), sb = std::sin(b), cw = std::cos(0.5 * B.dphi);
        const double r0 = (B.rin + vw0) / cw, r1 = (B.rin + vw0 + s->row_pitch) / cw, hw = 0.5 * s->vomitory_width;
        double lo[2] = {1e30, 1e30}, hi[2] = {-1e30, -1e30};
        for (int q = 0; q < 4; ++q) {
            const double r = (q & 1) ? r1 : r0, t = (q & 2) ? hw : -hw;
            const double x = r * cb - t * sb, y = r * sb + t * cb;
            lo[0] = std::min(lo[0], x); lo[1] = std::min(lo[1], y); hi[0] = std::max(hi[0], x); hi[1] = std::max(hi[1], y);
        }
        exitBoxes[4 * k] = float(lo[0]); exitBoxes[4 * k + 1] = float(lo[1]);
        exitBoxes[4 * k + 2] = float(hi[0]); exitBoxes[4 * k + 3] = float(hi[1]);
    }
    int e = s->sectors;
    for (int k = 0; k < s->sectors; ++k)
        if (B.exitSector[size_t(k)])
            bound(e++, k, -0.5 * s->perimeter_exit_width, 0.5 * s->perimeter_exit_width, B.outerW + B.wallT,
                  B.outerW + B.wallT + 3.0);
}

}  // namespace

extern "C" int swarm_bowl_fields(const SwarmBowlSpec* s, const SwarmVenue* v, float* wall, float* nav, float* floorH,
                                 float* speedF, uint8_t* mask, float* exitBoxes) {
    if (!validBowl(s) || !v || !wall || !nav || !floorH || !speedF || !mask) return SWARM_E_INVALID;
    const Bowl B(*s);
    const int wn = v->wall_nx, nn = v->nav_nx;
    parallelRows(v->wall_ny, [&](int j) {
        for (int i = 0; i < wn; ++i) {
            const double x = double(v->wall_origin_x) + i * double(v->wall_h), y = double(v->wall_origin_y) + j * double(v->wall_h);
            const size_t k = size_t(j) * size_t(wn) + size_t(i);
            double h, sp;
            B.floorAt(x, y, h, sp);
            wall[k] = float(B.sdf(x, y));
            floorH[k] = float(h);
            speedF[k] = float(sp);
        }
    });
    std::vector<uint8_t> kind;
    std::vector<float> speed;
    bowlNav(s, v, B, kind, speed, mask);
    if (const int rc = fastMarch(nn, v->nav_ny, v->nav_h, kind, speed.data(), nav); rc != SWARM_OK) return rc;
    fillBand(nn, v->nav_ny, v->nav_h, nav, BAND_SLOPE, BAND_REACH, kind.data());
    if (exitBoxes) bowlExitBoxes(s, B, exitBoxes);   // (the metrics' exit attribution)
    return SWARM_OK;
}

extern "C" int swarm_bowl_exit_fields(const SwarmBowlSpec* s, const SwarmVenue* v, float* fields, float* width, uint8_t* type) {
    if (!validBowl(s) || !v || !fields) return SWARM_E_INVALID;
    const int nExits = s->sectors + s->perimeter_exits;
    if (nExits < 1 || nExits > SWARM_CHOICE_MAX_EXITS) return SWARM_E_INVALID;
    const Bowl B(*s);
    std::vector<uint8_t> kind;
    std::vector<float> speed;
    bowlNav(s, v, B, kind, speed, nullptr);
    std::vector<float> boxes(size_t(4) * size_t(nExits));
    bowlExitBoxes(s, B, boxes.data());
    for (int e = 0; e < nExits; ++e) {   // the vomitories (avenues into the concourse), then the perimeter doors
        const bool vom = e < s->sectors;
        if (width) width[e] = vom ? s->vomitory_width : s->perimeter_exit_width;
        if (type) type[e] = vom ? 0 : 1;
    }
    return exitFields(v, kind, speed.data(), boxes.data(), nExits, fields, false, BAND_SLOPE);
}

extern "C" int swarm_spawn_bowl(const SwarmBowlSpec* sp, float jitter, uint64_t seed, float r_lo, float r_hi, float v_mean,
                                float v_sd, float v_lo, float v_hi, float* boids, float* radius, float* v0) {
    if (!validBowl(sp) || !boids || !radius || !v0) return SWARM_E_INVALID;
    const Bowl B(*sp);
    uint64_t s = seed;
    const double pi2 = 6.283185307179586;
    size_t i = 0;
    for (int k = 0; k < sp->sectors; ++k) {
        for (int row = 0; row < sp->rows; ++row) {
            for (int seat = 0; seat < sp->seats; ++seat, ++i) {
                const double u = -B.halfRow + (seat + 0.5) * sp->seat_width, w = (row + 0.5) * sp->row_pitch;
                const double jx = (2.0 * uniform01(s) - 1.0) * jitter, jy = (2.0 * uniform01(s) - 1.0) * jitter;
                const double rad = r_lo + (r_hi - r_lo) * uniform01(s);
                const double u1 = 1.0 - uniform01(s), u2 = uniform01(s);
                const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(pi2 * u2);
                const double v = std::min(std::max(v_mean + v_sd * z, double(v_lo)), double(v_hi));
                float* b = boids + i * 8;
                b[0] = float((B.rin + w) * B.c[size_t(k)] - u * B.sn[size_t(k)] + jx);
                b[1] = float((B.rin + w) * B.sn[size_t(k)] + u * B.c[size_t(k)] + jy);
                b[2] = float(row * double(sp->rise) + rad);
                b[3] = 1.0f;
                b[4] = b[5] = b[6] = b[7] = 0.0f;
                radius[i] = float(rad);
                v0[i] = float(v);
            }
        }
    }
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
