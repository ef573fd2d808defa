// ORACLE -- test infrastructure only. Nothing in the product links, loads or calls this file: the tests, the
// smoke check and bench.py's CPU-baseline leg use it as the checker of the CUDA step.
//
// A CPU restatement of SWARM's per-step crowd update (DedovSergei/swarm-crowd-simulation), written for this
// project from the reference's CPU port of its compute shaders, src/cpu_crowd_sim.cpp. Every function cites the
// reference lines it restates. Operation order follows the reference expression by expression (glm's vector
// arithmetic written out per component, glm::mix as x*(1-a)+y*a, glm::dot/length left to right), so that compiled
// with -ffp-contract=off it reproduces the reference bit for bit on the reference's own venue.
//
// Two venue kinds (the SwarmVenue format of include/swarm_cuda.h):
//   STADIUM  the reference's baked terrace: stadium.sdf, the analytic pitch fence, the egress router, model units,
//            uniform body. PINNED: it reproduces the unmodified reference (oracle/_ref, built from the reference's
//            own sources) bit for bit, checked by tests/test_oracle_pin.py on spawn and congested states.
//   GRID     plan venues on grids in SI units with per-agent radius and desired speed: the wall query of the
//            reference's analytic-venue branch (cpu_crowd_sim.cpp clearWalls / wallPlaneProbe "seated" paths)
//            over a horizontal wall SDF, e_goal = -grad D / |grad D| of a geodesic distance grid. The reference has
//            no such venue: this branch is pinned only through the shared skeleton (predict, projection, final
//            pass) that the stadium pin covers.
//
// The state is the reference's GpuBoid array (8 floats per agent), the sort is the reference's SortMode::Counting
// (stable by agent id within a cell, inactive agents at the tail).

#include "swarm_oracle.hpp"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace oracle {
namespace {

constexpr uint32_t INACTIVE_CELL = 0xFFFFFFFFu;
constexpr float PLANE_WALL = 1.0f, PLANE_GROUNDED = 2.0f;
constexpr float WALL_NONE = 1e9f;
// the queue-aware exit choice's constants (include/swarm/sim_params.hpp:412-427, include/swarm/exit_choice.hpp:121-137;
// the queue-ahead bins 0.5 m on SI venues)
constexpr double CHOICE_T_S = 3.0;
constexpr float CHOICE_REL_MARGIN = 0.10f, CHOICE_ABS_MARGIN_S = 5.0f, CHOICE_SWITCH_SHARE = 0.10f;
constexpr uint32_t CHOICE_MIN_SWITCHES = 1;
constexpr int CHOICE_GAIN_BINS = 256, CHOICE_AHEAD_BINS = 1024, CHOICE_STRIDE = 64;
constexpr float CHOICE_S_PER_M = float(1.0 / double(1.34f));   // 1 / V_FREE_M_S

// ContactBits (include/swarm/cpu_crowd_sim.hpp:52-61)
enum : uint8_t { C_EXIT = 1, C_FENCE_CCD = 2, C_FENCE = 4, C_FLOOR = 8, C_WALL = 16, C_AGENT = 32, C_SWEEP = 64, C_STEP_UP = 128 };

// ---- small vector arithmetic in glm's operation order ----
template <class T> struct V2 { T x, y; };
template <class T> struct V3 { T x, y, z; };
template <class T> struct V4 { T x, y, z, w; };
template <class T> inline V2<T> v2(T x, T y) { return {x, y}; }
template <class T> inline V2<T> operator+(V2<T> a, V2<T> b) { return {a.x + b.x, a.y + b.y}; }
template <class T> inline V2<T> operator-(V2<T> a, V2<T> b) { return {a.x - b.x, a.y - b.y}; }
template <class T> inline V2<T> operator-(V2<T> a) { return {-a.x, -a.y}; }
template <class T> inline V2<T> operator*(V2<T> a, T s) { return {a.x * s, a.y * s}; }
template <class T> inline V2<T> operator*(T s, V2<T> a) { return {s * a.x, s * a.y}; }
template <class T> inline V2<T> operator*(V2<T> a, V2<T> b) { return {a.x * b.x, a.y * b.y}; }
template <class T> inline V2<T> operator/(V2<T> a, T s) { return {a.x / s, a.y / s}; }
template <class T> inline bool operator==(V2<T> a, V2<T> b) { return a.x == b.x && a.y == b.y; }
template <class T> inline bool operator!=(V2<T> a, V2<T> b) { return !(a == b); }
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> inline T dot(V2<T> a, V2<T> b) { return a.x * b.x + a.y * b.y; }
template <class T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline T length(V2<T> a) { return std::sqrt(dot(a, a)); }
template <class T> inline T length(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> inline T mix(T a, T b, T t) { return a * (T(1) - t) + b * t; }
template <class T> inline V2<T> mix(V2<T> a, V2<T> b, T t) { return {mix(a.x, b.x, t), mix(a.y, b.y, t)}; }
template <class T> inline V2<T> xy(V3<T> a) { return {a.x, a.y}; }
template <class T> inline V2<T> xy(V4<T> a) { return {a.x, a.y}; }
template <class T> inline V3<T> xyz(V4<T> a) { return {a.x, a.y, a.z}; }
template <class T> inline void setXY(V3<T>& v, V2<T> a) { v.x = a.x; v.y = a.y; }

using F2 = V2<float>;
using F3 = V3<float>;
using F4 = V4<float>;

struct Boid { F4 pos, vel; };   // GpuBoid (include/swarm/gpu_types.hpp:17-20)
static_assert(sizeof(Boid) == 32, "GpuBoid layout");
struct Pair { uint32_t key, id; };
struct Cell { uint32_t start, count; };

// physics.comp safeNormalize (cpu_crowd_sim.cpp:94-95)
template <class T> inline V2<T> safeNormalize(V2<T> v, T eps) { T l = length(v); return l > eps ? v / l : V2<T>{T(0), T(0)}; }
template <class T> inline V3<T> safeNormalize(V3<T> v, T eps) {
    T l = length(v);
    return l > eps ? V3<T>{v.x / l, v.y / l, v.z / l} : V3<T>{T(0), T(0), T(0)};
}

// lowbias32 (cpu_crowd_sim.cpp:120-125)
inline uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du;
    x ^= x >> 15; x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// cpu_crowd_sim.cpp:127-133: the separation direction of a stacked pair
inline F2 pairDirection(uint32_t self, uint32_t other, float hashToRadians) {
    uint32_t lo = std::min(self, other), hi = std::max(self, other);
    float angle = float(hash32(hash32(lo) ^ hi)) * hashToRadians;
    F2 dir{std::cos(angle), std::sin(angle)};
    return self == lo ? dir : -dir;
}

// cpu_crowd_sim.cpp:135-143, with the support radius rsep (uniform: R_SEP) of the pair
inline F2 separationForce(const SwarmParams& P, F3 offset, uint32_t self, uint32_t other, float rsep, float rsep2) {
    float d2 = dot(offset, offset);
    if (d2 >= rsep2) return {0.0f, 0.0f};
    float w = 1.0f - std::sqrt(d2) / rsep;
    float magnitude = P.k_sep * w * w;
    float dxy2 = dot(xy(offset), xy(offset));
    if (dxy2 <= P.stacked_xy2) return magnitude * pairDirection(self, other, P.hash_to_radians);
    return magnitude * xy(offset) * (1.0f / std::sqrt(dxy2));
}

// cpu_crowd_sim.cpp:145-152, with the contact distance dc (uniform: BODY_DIAM) of the pair
inline F2 contactCorrection(const SwarmParams& P, F3 offset, uint32_t self, uint32_t other, float dc, float dc2) {
    float dxy2 = dot(xy(offset), xy(offset));
    if (std::abs(offset.z) >= dc || dxy2 >= dc2) return {0.0f, 0.0f};
    float dxy = std::sqrt(dxy2);
    float shift = 0.5f * (dc - dxy);
    if (dxy2 <= P.stacked_xy2) return shift * pairDirection(self, other, P.hash_to_radians);
    return shift * (xy(offset) / dxy);
}

// ================================================================================================================
// STADIUM venue: the baked terrace of the reference
// ================================================================================================================
struct Stadium {
    const SwarmParams& P;
    const float* texels;   // sdf_res^3, [x][y][z]
    int res;
    F3 sdfMin;
    float spacing, invSpacing;
    F2 fenceC, fenceMid;
    float domainMin, domainSpan, domainMax, exitDepth, exitMaxZ;
    int gridRes;

    float texel(int x, int y, int z) const { return texels[(size_t(x) * size_t(res) + size_t(y)) * size_t(res) + size_t(z)]; }

    // src/sdf.cpp:21-43 sampleSDF: the exact-weight trilinear sampler (the CPU's map())
    float map(F3 pos) const {
        F3 uvw{(1.5f + (pos.x - sdfMin.x) / spacing) / float(res), (1.5f + (pos.y - sdfMin.y) / spacing) / float(res),
               (1.5f + (pos.z - sdfMin.z) / spacing) / float(res)};
        if (uvw.x < 0.0f || uvw.y < 0.0f || uvw.z < 0.0f || uvw.x > 1.0f || uvw.y > 1.0f || uvw.z > 1.0f) return 1.0f;
        F3 t{uvw.x * float(res) - 0.5f, uvw.y * float(res) - 0.5f, uvw.z * float(res) - 0.5f};
        F3 base{std::floor(t.x), std::floor(t.y), std::floor(t.z)};
        F3 f{t.x - base.x, t.y - base.y, t.z - base.z};
        auto at = [this](int x, int y, int z) {
            x = std::clamp(x, 0, res - 1); y = std::clamp(y, 0, res - 1); z = std::clamp(z, 0, res - 1);
            return texel(x, y, z);
        };
        int x0 = int(base.x), y0 = int(base.y), z0 = int(base.z);
        float c00 = mix(at(x0, y0, z0), at(x0 + 1, y0, z0), f.x);
        float c10 = mix(at(x0, y0 + 1, z0), at(x0 + 1, y0 + 1, z0), f.x);
        float c01 = mix(at(x0, y0, z0 + 1), at(x0 + 1, y0, z0 + 1), f.x);
        float c11 = mix(at(x0, y0 + 1, z0 + 1), at(x0 + 1, y0 + 1, z0 + 1), f.x);
        return mix(mix(c00, c10, f.y), mix(c01, c11, f.y), f.z);
    }

    // cpu_crowd_sim.cpp:255-261
    float columnLevel(int i0x, int i0y, F2 w, int k) const {
        k = std::clamp(k, 0, res - 1);
        float c0 = mix(texel(i0x, i0y, k), texel(i0x + 1, i0y, k), w.x);
        float c1 = mix(texel(i0x, i0y + 1, k), texel(i0x + 1, i0y + 1, k), w.x);
        return mix(c0, c1, w.y);
    }

    F3 toTex(F3 p) const {   // 1 + (p - U_SDF_MIN) * U_SDF_INV_SPACING
        return {1.0f + (p.x - sdfMin.x) * invSpacing, 1.0f + (p.y - sdfMin.y) * invSpacing, 1.0f + (p.z - sdfMin.z) * invSpacing};
    }

    // cpu_crowd_sim.cpp:263-287 mapExactGrad: vec4(gradient, value)
    F4 mapExactGrad(F3 p) const {
        F3 f = toTex(p);
        const float hiLim = float(res) - 0.5f;
        bool outside = f.x < -0.5f || f.y < -0.5f || f.z < -0.5f || f.x > hiLim || f.y > hiLim || f.z > hiLim;
        int ix = std::clamp(int(std::floor(f.x)), 0, res - 2);
        int iy = std::clamp(int(std::floor(f.y)), 0, res - 2);
        int iz = std::clamp(int(std::floor(f.z)), 0, res - 2);
        F3 w{f.x - float(ix), f.y - float(iy), f.z - float(iz)};
        float c000 = texel(ix, iy, iz), c100 = texel(ix + 1, iy, iz), c010 = texel(ix, iy + 1, iz), c110 = texel(ix + 1, iy + 1, iz);
        float c001 = texel(ix, iy, iz + 1), c101 = texel(ix + 1, iy, iz + 1), c011 = texel(ix, iy + 1, iz + 1);
        float c111 = texel(ix + 1, iy + 1, iz + 1);
        float x00 = mix(c000, c100, w.x), x10 = mix(c010, c110, w.x);
        float x01 = mix(c001, c101, w.x), x11 = mix(c011, c111, w.x);
        float y0 = mix(x00, x10, w.y), y1 = mix(x01, x11, w.y);
        float gx = mix(mix(c100 - c000, c110 - c010, w.y), mix(c101 - c001, c111 - c011, w.y), w.z);
        float gy = mix(x10 - x00, x11 - x01, w.z);
        float gz = y1 - y0;
        if (outside) return {0.0f, 0.0f, 0.0f, 1.0f};
        return {gx * invSpacing, gy * invSpacing, gz * invSpacing, mix(y0, y1, w.z)};
    }

    // cpu_crowd_sim.cpp:289-316 floorUnderReach
    bool floorUnderReach(F3 c, float zFrom, float down, float& zFloor) const {
        zFloor = 0.0f;
        F3 f = toTex(c);
        const float hiLim = float(res) - 1.0f;
        if (f.x < 0.0f || f.y < 0.0f || f.x > hiLim || f.y > hiLim) return false;
        int i0x = std::min(int(std::floor(f.x)), res - 2), i0y = std::min(int(std::floor(f.y)), res - 2);
        F2 w{f.x - float(i0x), f.y - float(i0y)};
        int k = int(std::floor(f.z));
        float vLo = columnLevel(i0x, i0y, w, k), vHi = columnLevel(i0x, i0y, w, k + 1);
        bool inSolid = mix(vLo, vHi, f.z - float(k)) <= 0.0f;
        float fLimit = f.z + (inSolid ? std::max(zFrom, c.z) + P.body_radius - c.z : -down) * invSpacing;
        for (int cell = 0; cell < P.floor_search_cells; ++cell) {
            float fEnd = inSolid ? std::min(float(k + 1), fLimit) : std::max(float(k), fLimit);
            float vEnd = mix(vLo, vHi, fEnd - float(k));
            if (inSolid ? vEnd > 0.0f : vEnd <= 0.0f) {
                float fRoot = float(k) + vLo / (vLo - vHi);
                zFloor = sdfMin.z + (fRoot - 1.0f) / invSpacing;
                return true;
            }
            if (fEnd == fLimit) return false;
            if (inSolid) { ++k; vLo = vHi; vHi = columnLevel(i0x, i0y, w, k + 1); }
            else         { --k; vHi = vLo; vLo = columnLevel(i0x, i0y, w, k); }
        }
        return false;
    }

    // src/sdf.cpp:45-57, 64-82: the analytic pitch fence
    static float sdBox2(F2 p, F2 half) {
        F2 q{std::abs(p.x) - half.x, std::abs(p.y) - half.y};
        F2 qp{std::max(q.x, 0.0f), std::max(q.y, 0.0f)};
        return length(qp) + std::min(std::max(q.x, q.y), 0.0f);
    }
    static F2 sdBox2Grad(F2 p, F2 half) {
        F2 q{std::abs(p.x) - half.x, std::abs(p.y) - half.y};
        F2 s{p.x < 0.0f ? -1.0f : 1.0f, p.y < 0.0f ? -1.0f : 1.0f};
        F2 g;
        if (std::max(q.x, q.y) > 0.0f) {
            F2 qp{std::max(q.x, 0.0f), std::max(q.y, 0.0f)};
            g = qp / length(qp);
        } else {
            g = q.x > q.y ? F2{1.0f, 0.0f} : F2{0.0f, 1.0f};
        }
        return s * g;
    }
    float sdFence(F3 p) const { return std::abs(sdBox2(xy(p) - fenceC, fenceMid)) - P.fence_half_thk_coll; }
    F2 sdFenceGradient(F3 p) const {
        F2 rel = xy(p) - fenceC;
        float box = sdBox2(rel, fenceMid);
        return (box < 0.0f ? -1.0f : 1.0f) * sdBox2Grad(rel, fenceMid);
    }

    // cpu_crowd_sim.cpp:99-116 fenceCCD
    bool fenceCCD(F3 pOld, F3& pNew, F3& vel) const {
        float sOld = sdBox2(xy(pOld) - fenceC, fenceMid);
        float sNew = sdBox2(xy(pNew) - fenceC, fenceMid);
        if (sOld * sNew >= 0.0f) return false;
        float side = sOld > 0.0f ? 1.0f : -1.0f;
        float lo = 0.0f;
        if (side * sOld > P.fence_half_thk_coll) {
            float hi = 1.0f;
            for (int i = 0; i < P.fence_ccd_bisections; ++i) {
                float t = 0.5f * (lo + hi);
                if (side * sdBox2(mix(xy(pOld), xy(pNew), t) - fenceC, fenceMid) > P.fence_half_thk_coll) lo = t;
                else hi = t;
            }
        }
        setXY(pNew, mix(xy(pOld), xy(pNew), lo));
        F2 n = sdFenceGradient(pNew);
        float vn = dot(xy(vel), n);
        if (vn < 0.0f) setXY(vel, xy(vel) - n * vn);
        return true;
    }

    // cpu_crowd_sim.cpp:154-172 egressTarget / egressDirection
    F2 goal(F3 p) const {
        F2 s{p.x < 0.0f ? -1.0f : 1.0f, p.y < 0.0f ? -1.0f : 1.0f};
        F2 a{std::abs(p.x), std::abs(p.y)};
        bool alongX = a.y >= a.x;
        float lat = alongX ? a.x : a.y;
        float dep = alongX ? a.y : a.x;
        F2 t;
        if (lat < P.avenue_half && dep >= P.walkway_min) t = {0.0f, P.avenue_target_depth};
        else if (dep >= P.walkway_min && dep < P.walkway_max) t = {0.0f, P.walkway_centre};
        else if (dep >= P.walkway_max && lat < P.aisle_max) t = {P.aisle_centre, P.walkway_centre};
        else if (dep >= P.walkway_max) t = {P.aisle_centre, dep};
        else t = {0.0f, P.pitch_recovery_depth};
        F2 target = alongX ? s * t : s * F2{t.y, t.x};
        F2 toTarget = target - xy(p);
        return length(toTarget) > P.goal_deadzone ? safeNormalize(toTarget, P.safe_eps) : F2{0.0f, 0.0f};
    }

    // cpu_crowd_sim.cpp:662-668 exit test
    bool exits(F4 p) const {
        float m = std::max(std::abs(p.x), std::abs(p.y));
        return (m > exitDepth && p.z < exitMaxZ) || m > domainMax;
    }

    // cpu_crowd_sim.cpp:312-321 calcGradient / calcNormal, 323-332 sceneDist / sceneNormal
    F3 calcGradient(F3 p) const {
        const F3 kxyy{1.0f, -1.0f, -1.0f}, kyyx{-1.0f, -1.0f, 1.0f}, kyxy{-1.0f, 1.0f, -1.0f}, kxxx{1.0f, 1.0f, 1.0f};
        const float h = P.obstacle_grad_h;
        F3 a = kxyy * map(p + kxyy * h), b = kyyx * map(p + kyyx * h), c = kyxy * map(p + kyxy * h), d = kxxx * map(p + kxxx * h);
        return (a + b + c + d) * P.obstacle_grad_scale;
    }
    float sceneDist(F3 p, bool& fenceActive) const {
        float dStadium = map(p);
        float dFence = sdFence(p) + P.body_radius;
        fenceActive = dFence < dStadium;
        return fenceActive ? dFence : dStadium;
    }
    F2 sceneNormal(F3 p, bool fenceActive) const {
        return fenceActive ? sdFenceGradient(p) : xy(safeNormalize(calcGradient(p), P.safe_eps));
    }

    bool restOnFloor(F3& np, F3& nv, float zFrom) const {   // cpu_crowd_sim.cpp:334-342
        float zFloor;
        if (floorUnderReach(np, zFrom, P.body_radius, zFloor) && np.z < zFloor + P.body_radius) {
            np.z = zFloor + P.body_radius;
            nv.z = 0.0f;
            return true;
        }
        return false;
    }
    bool settleOnFloor(F3& np, F3& nv, float zFrom) const {   // cpu_crowd_sim.cpp:344-352
        float zFloor;
        if (floorUnderReach(np, zFrom, P.floor_settle_reach, zFloor)) {
            np.z = zFloor + P.body_radius;
            nv.z = 0.0f;
            return true;
        }
        return false;
    }

    // cpu_crowd_sim.cpp:174-184 rootStep / newtonStep; br = (a, f(a), b, f(b))
    static float rootStep(F4& br, float t, F4 g, F3 u) {
        if (g.w > 0.0f) { br.x = t; br.y = g.w; } else { br.z = t; br.w = g.w; }
        float du = dot(F3{g.x, g.y, g.z}, u);
        float tn = du < 0.0f ? t - g.w / du : -1.0f;
        return tn > br.x && tn < br.z ? tn : (br.x * br.w - br.z * br.y) / (br.w - br.y);
    }
    static float newtonStep(float t, F4 g, F3 u) {
        float du = dot(F3{g.x, g.y, g.z}, u);
        return du < 0.0f ? t - g.w / du : t;
    }

    // cpu_crowd_sim.cpp:354-382 wallContact
    float wallContact(F3 np, float fc, F3 u, float fr, float reach, F2& away) const {
        F4 br{0.0f, fc, reach, fr};
        float t = reach * fc / (fc - fr);
        F4 g{0.0f, 0.0f, 0.0f, 0.0f};
        for (int i = 0; i < P.wall_root_steps; ++i) {
            g = mapExactGrad(np + u * t);
            t = rootStep(br, t, g, u);
        }
        bool wall = g.z <= P.wall_max_nz * length(F3{g.x, g.y, g.z});
        float e = wall ? t : 1e9f;
        away = F2{-u.x, -u.y};
        F2 n = safeNormalize(F2{g.x, g.y}, P.safe_eps);
        F3 u2{-n.x, -n.y, 0.0f};
        float t2 = 0.0f, t3 = t * dot(u, u2);
        F4 g2{0.0f, 0.0f, 0.0f, 0.0f};
        for (int i = 0; i < P.wall_recast_steps; ++i) {
            t2 = t3;
            g2 = mapExactGrad(np + u2 * t2);
            t3 = newtonStep(t2, g2, u2);
        }
        bool ok = wall && dot(F3{g2.x, g2.y, g2.z}, u2) < 0.0f && std::abs(t3 - t2) < P.wall_recast_tol && t3 > 0.0f &&
                  g2.z <= P.wall_max_nz * length(F3{g2.x, g2.y, g2.z});
        if (ok && t3 < e) { e = t3; away = n; }
        return e;
    }

    // cpu_crowd_sim.cpp:384-441 clearWalls (baked branch)
    bool clearWalls(F3& np, F3& nv, F3& wall) const {
        bool moved = false;
        wall = {0.0f, 0.0f, 0.0f};
        for (int pass = 0; pass < P.wall_passes; ++pass) {
            bool nearFence = sdFence(np) < P.feeler_reach;
            float fc = map(np);
            float fr1 = 0.0f, fr2 = 0.0f;
            int i1 = -1, i2 = -1;
            for (int i = 0; i < P.feeler_count; ++i) {
                F3 f = np + F3{P.feeler_off[i][0], P.feeler_off[i][1], 0.0f};
                float v = map(f);
                if (nearFence && sdFence(f) < 0.0f) v = 1.0f;
                if (v < fr1)      { fr2 = fr1; i2 = i1; fr1 = v; i1 = i; }
                else if (v < fr2) { fr2 = v; i2 = i; }
            }
            if (i1 < 0) break;
            F2 hNorm;
            float clearance;
            if (fc > 0.0f) {
                clearance = wallContact(np, fc, F3{P.feeler_dir[i1][0], P.feeler_dir[i1][1], 0.0f}, fr1, P.feeler_reach, hNorm);
                if (i2 >= 0) {
                    F2 h2;
                    float c2 = wallContact(np, fc, F3{P.feeler_dir[i2][0], P.feeler_dir[i2][1], 0.0f}, fr2, P.feeler_reach, h2);
                    if (c2 < clearance) { clearance = c2; hNorm = h2; }
                }
            } else {
                F4 g = mapExactGrad(np);
                hNorm = safeNormalize(F2{g.x, g.y}, P.safe_eps);
                clearance = g.w / std::max(length(F2{g.x, g.y}), P.centre_grad_min);
            }
            if (clearance >= P.body_radius) {
                if (clearance < 1e9f) wall = {hNorm.x, hNorm.y, clearance - P.body_radius};
                break;
            }
            setXY(np, xy(np) + hNorm * (P.body_radius - clearance));
            moved = true;
            wall = {hNorm.x, hNorm.y, 0.0f};
            float vDotN = dot(xy(nv), hNorm);
            if (vDotN < 0.0f) setXY(nv, xy(nv) - hNorm * vDotN);
        }
        return moved;
    }

    // cpu_crowd_sim.cpp:443-461 wallPlaneProbe (baked branch)
    F3 wallPlaneProbe(F3 np) const {
        bool nearFence = sdFence(np) < P.plane_probe_reach;
        float fc = map(np);
        float fr = 0.0f;
        int i1 = -1;
        for (int i = 0; i < P.feeler_count; ++i) {
            F3 f = np + F3{P.probe_off[i][0], P.probe_off[i][1], 0.0f};
            float v = map(f);
            if (nearFence && sdFence(f) < 0.0f) v = 1.0f;
            if (v < fr) { fr = v; i1 = i; }
        }
        if (i1 < 0 || fc <= 0.0f) return {0.0f, 0.0f, 0.0f};
        F2 away;
        float c = wallContact(np, fc, F3{P.feeler_dir[i1][0], P.feeler_dir[i1][1], 0.0f}, fr, P.plane_probe_reach, away);
        return c < 1e9f ? F3{away.x, away.y, std::max(c - P.body_radius, 0.0f)} : F3{0.0f, 0.0f, 0.0f};
    }

    bool bakedSolid(F3 p) const { return sdFence(p) >= 0.0f && mapExactGrad(p).w <= 0.0f; }   // cpu_crowd_sim.cpp:463

    // cpu_crowd_sim.cpp:465-479 sweepBack
    bool sweepBack(F3 pOld, F3& np, F3& nv) const {
        if (!bakedSolid(np)) return false;
        float lo = 0.0f, hi = 1.0f;
        if (!bakedSolid(F3{np.x, np.y, pOld.z})) lo = 1.0f;
        for (int i = 0; i < P.sweep_bisections; ++i) {
            float t = 0.5f * (lo + hi);
            F2 m = mix(xy(pOld), xy(np), t);
            if (bakedSolid(F3{m.x, m.y, pOld.z})) hi = t;
            else lo = t;
        }
        F2 d = safeNormalize(xy(np) - xy(pOld), P.safe_eps);
        F2 m = mix(xy(pOld), xy(np), lo);
        np = {m.x, m.y, pOld.z};
        float vd = dot(xy(nv), d);
        if (vd > 0.0f) setXY(nv, xy(nv) - d * vd);
        nv.z = 0.0f;
        return true;
    }

    // cpu_crowd_sim.cpp:483-514 resolveStatic
    bool resolveStatic(F3 pOld, F3& np, F3& nv, bool settle, F3& wall, uint8_t& contact) const {
        if (fenceCCD(pOld, np, nv)) contact |= C_FENCE_CCD;
        float dFence = sdFence(np);
        if (dFence < 0.0f) {
            F2 n = sdFenceGradient(np);
            setXY(np, xy(np) - n * dFence);
            float vDotN = dot(xy(nv), n);
            if (vDotN < 0.0f) setXY(nv, xy(nv) - n * vDotN);
            contact |= C_FENCE;
        }
        bool grounded = settle ? settleOnFloor(np, nv, pOld.z) : restOnFloor(np, nv, pOld.z);
        if (!grounded && sweepBack(pOld, np, nv)) {
            contact |= C_SWEEP;
            grounded = restOnFloor(np, nv, pOld.z);
        }
        if (grounded) contact |= C_FLOOR;
        const bool walls = clearWalls(np, nv, wall);
        if (walls) {
            contact |= C_WALL;
            if (grounded) {
                if (settleOnFloor(np, nv, pOld.z)) contact |= C_FLOOR;
                F3 w2;
                const bool again = clearWalls(np, nv, w2);
                if (w2.x != 0.0f || w2.y != 0.0f) wall = w2;
                if (again && restOnFloor(np, nv, pOld.z)) contact |= C_FLOOR;
            } else if (restOnFloor(np, nv, pOld.z)) {
                contact |= C_FLOOR;
            }
        }
        return grounded;
    }

    // cpu_crowd_sim.cpp:518-544 stepUpWindow
    int stepUpWindow(F2 pxy, float f0, F4& g) const {
        g = {0.0f, 0.0f, 1.0f, 0.0f};
        F3 f = toTex(F3{pxy.x, pxy.y, f0});
        const float hiLim = float(res) - 1.0f;
        if (f.x < 0.0f || f.y < 0.0f || f.x > hiLim || f.y > hiLim) return 0;
        int i0x = std::min(int(std::floor(f.x)), res - 2), i0y = std::min(int(std::floor(f.y)), res - 2);
        F2 w{f.x - float(i0x), f.y - float(i0y)};
        float fLo = f.z + P.step_up_tol * invSpacing, fHi = f.z + P.max_step_up * invSpacing;
        int k = int(std::floor(fHi));
        float a = columnLevel(i0x, i0y, w, k), b = columnLevel(i0x, i0y, w, k + 1);
        if (mix(a, b, fHi - float(k)) <= 0.0f) {
            g = mapExactGrad(F3{pxy.x, pxy.y, sdfMin.z + (fHi - 1.0f) / invSpacing});
            return 2;
        }
        for (int cell = 0; cell < 2; ++cell) {
            float fBot = std::max(float(k), fLo);
            if (mix(a, b, fBot - float(k)) <= 0.0f) {
                float fRoot = float(k) + a / (a - b);
                g = mapExactGrad(F3{pxy.x, pxy.y, sdfMin.z + (fRoot - 1.0f) / invSpacing});
                return 1;
            }
            if (fBot == fLo) return 0;
            --k; b = a; a = columnLevel(i0x, i0y, w, k);
        }
        return 0;
    }
    bool stepUpBlocked(int r, F4 g, F2 dir, bool end) const {   // cpu_crowd_sim.cpp:546-549
        if (r == 2) return end;
        return r == 1 && dot(F2{g.x, g.y}, dir) < 0.0f && g.z <= P.wall_max_nz * length(F3{g.x, g.y, g.z});
    }
    // cpu_crowd_sim.cpp:555-580 stepUpScan
    float stepUpScan(F2 p0, F2 p1, float f0, F2& n) const {
        n = {0.0f, 0.0f};
        F2 d = p1 - p0;
        float len = length(d);
        F2 dir = len > 0.0f ? d / len : F2{0.0f, 0.0f};
        int ns = std::clamp(int(std::ceil(len / P.step_up_sample)), 1, P.step_up_max_samples);
        int lastOk = 0;
        bool blocked = false;
        for (int i = 1; i <= ns; ++i) {
            F4 g;
            int r = stepUpWindow(mix(p0, p1, float(i) / float(ns)), f0, g);
            if (stepUpBlocked(r, g, dir, i == ns)) { blocked = true; n = safeNormalize(F2{g.x, g.y}, P.safe_eps); break; }
            if (r != 2) lastOk = i;
        }
        if (!blocked) return 1.0f;
        float lo = float(lastOk) / float(ns), hi = float(lastOk + 1) / float(ns);
        for (int i = 0; i < P.step_up_bisections; ++i) {
            float t = 0.5f * (lo + hi);
            F4 g;
            int r = stepUpWindow(mix(p0, p1, t), f0, g);
            if (stepUpBlocked(r, g, dir, true)) { hi = t; n = safeNormalize(F2{g.x, g.y}, P.safe_eps); }
            else lo = t;
        }
        return lo;
    }
    // cpu_crowd_sim.cpp:583-613 limitStepUp (baked branch)
    bool limitStepUp(F3 pOld, F3& np, F3& nv) const {
        float f0;
        if (!floorUnderReach(pOld, pOld.z, P.step_up_floor_reach, f0)) f0 = pOld.z - P.step_up_floor_reach;
        F2 n;
        float t = stepUpScan(xy(pOld), xy(np), f0, n);
        if (t >= 1.0f) return false;
        F2 q = mix(xy(pOld), xy(np), t);
        F2 rest = xy(np) - q;
        F2 tangent = rest - n * dot(rest, n);
        float lt = length(tangent);
        if (lt > 0.0f) {
            for (int k = 0; k < P.step_up_slide_tries; ++k) {
                F2 slide = q + tangent * P.step_up_slide[k][0] + n * (lt * P.step_up_slide[k][1]);
                F2 n2;
                if (sdFence(F3{slide.x, slide.y, 0.0f}) >= 0.0f && stepUpScan(q, slide, f0, n2) >= 1.0f) { q = slide; break; }
            }
        }
        float vn = dot(xy(nv), n);
        if (vn < 0.0f) setXY(nv, xy(nv) - n * vn);
        float zFloor;
        if (floorUnderReach(F3{q.x, q.y, pOld.z}, pOld.z, P.floor_settle_reach, zFloor)) {
            np = {q.x, q.y, zFloor + P.body_radius};
            nv.z = 0.0f;
        } else {
            np = {q.x, q.y, std::min(np.z, pOld.z)};
        }
        return true;
    }

    // projection's fence bound (cpu_crowd_sim.cpp:813-814)
    void fenceProject(F3& q) const {
        float dFence = sdFence(q);
        if (dFence < 0.0f) setXY(q, xy(q) - sdFenceGradient(q) * dFence);
    }
};

// ================================================================================================================
// GRID venue (SI units, per-agent radius): the wall query, floor and nav field on grids
// ================================================================================================================
struct GridVenue {
    const SwarmParams& P;
    const SwarmVenue& V;
    float wallInvH, navInvH;
    float domMinX, domMinY, domMaxX, domMaxY;

    // Bilinear value and gradient of the wall SDF at xy: (n away from the wall, distance); (0, 0, WALL_NONE) when
    // the distance is at least `reach` or xy lies outside the field (the analytic venue's wall query, cpu_crowd_sim.cpp:386-399)
    F3 wall(F2 p, float reach) const {
        float fx = (p.x - V.wall_origin_x) * wallInvH, fy = (p.y - V.wall_origin_y) * wallInvH;
        if (!(fx >= 0.0f && fy >= 0.0f && fx <= float(V.wall_nx - 1) && fy <= float(V.wall_ny - 1))) return {0.0f, 0.0f, WALL_NONE};
        int ix = std::min(int(std::floor(fx)), V.wall_nx - 2), iy = std::min(int(std::floor(fy)), V.wall_ny - 2);
        float wx = fx - float(ix), wy = fy - float(iy);
        const float* W = V.wall_sdf;
        size_t r0 = size_t(iy) * size_t(V.wall_nx) + size_t(ix), r1 = r0 + size_t(V.wall_nx);
        float c00 = W[r0], c10 = W[r0 + 1], c01 = W[r1], c11 = W[r1 + 1];
        float d = mix(mix(c00, c10, wx), mix(c01, c11, wx), wy);
        if (d >= reach) return {0.0f, 0.0f, WALL_NONE};
        F2 g{mix(c10 - c00, c11 - c01, wy) * wallInvH, mix(c01 - c00, c11 - c10, wx) * wallInvH};
        F2 n = safeNormalize(g, P.safe_eps);
        return {n.x, n.y, d};
    }
    float wallDist(F2 p) const {
        F3 w = wall(p, WALL_NONE);
        return w.z;
    }
    int floorNode(F2 p, size_t& idx) const {
        float fx = (p.x - V.wall_origin_x) * wallInvH + 0.5f, fy = (p.y - V.wall_origin_y) * wallInvH + 0.5f;
        int ix = std::clamp(int(std::floor(fx)), 0, V.wall_nx - 1), iy = std::clamp(int(std::floor(fy)), 0, V.wall_ny - 1);
        idx = size_t(iy) * size_t(V.wall_nx) + size_t(ix);
        return 0;
    }
    float floorHeight(F2 p) const {
        if (!V.floor_height) return 0.0f;
        size_t i; floorNode(p, i);
        return V.floor_height[i];
    }
    float speedFactor(F2 p) const {
        if (!V.speed_factor) return 1.0f;
        size_t i; floorNode(p, i);
        return V.speed_factor[i];
    }
    // The 3D distance of the obstacle avoidance and the static sweep: the walls and the floor
    float map(F3 p) const { return std::min(wallDist(xy(p)), p.z - floorHeight(xy(p))); }

    // e_goal: -grad D / |grad D| of the bilinear interpolant of the distance field (the nearest exit's, or D = one
    // exit's own field on the same grid: the queue-aware exit choice)
    F2 goal(F3 p) const { return goalIn(V.nav_dist, p); }
    F2 goalIn(const float* D, F3 p) const {
        float fx = (p.x - V.nav_origin_x) * navInvH, fy = (p.y - V.nav_origin_y) * navInvH;
        fx = std::clamp(fx, 0.0f, float(V.nav_nx - 1));
        fy = std::clamp(fy, 0.0f, float(V.nav_ny - 1));
        int ix = std::min(int(std::floor(fx)), V.nav_nx - 2), iy = std::min(int(std::floor(fy)), V.nav_ny - 2);
        float wx = fx - float(ix), wy = fy - float(iy);
        size_t r0 = size_t(iy) * size_t(V.nav_nx) + size_t(ix), r1 = r0 + size_t(V.nav_nx);
        float d00 = D[r0], d10 = D[r0 + 1], d01 = D[r1], d11 = D[r1 + 1];
        F2 g{mix(d10 - d00, d11 - d01, wy), mix(d01 - d00, d11 - d10, wx)};
        return safeNormalize(F2{-g.x, -g.y}, P.safe_eps);
    }

    bool exits(F4 p) const {
        bool outDomain = p.x < domMinX || p.x > domMaxX || p.y < domMinY || p.y > domMaxY;
        if (V.exit_mask) {   // the exit mask: the nav node nearest to p
            float fx = (p.x - V.nav_origin_x) * navInvH + 0.5f, fy = (p.y - V.nav_origin_y) * navInvH + 0.5f;
            int ix = std::clamp(int(std::floor(fx)), 0, V.nav_nx - 1), iy = std::clamp(int(std::floor(fy)), 0, V.nav_ny - 1);
            return outDomain || V.exit_mask[size_t(iy) * size_t(V.nav_nx) + size_t(ix)] != 0;
        }
        bool out = p.x < V.exit_lo_x || p.x > V.exit_hi_x || p.y < V.exit_lo_y || p.y > V.exit_hi_y;
        return (out && p.z < V.exit_max_z) || outDomain;
    }

    // The analytic venue's floor contact (cpu_crowd_sim.cpp:291-297), radius r
    bool floorUnderReach(F3 c, float zFrom, float down, float r, float& zFloor) const {
        const float h = floorHeight(xy(c));
        zFloor = h;
        if (c.z <= h) return h <= std::max(zFrom, c.z) + r;
        return h >= c.z - down;
    }
    bool restOnFloor(F3& np, F3& nv, float zFrom, float r) const {
        float zFloor;
        if (floorUnderReach(np, zFrom, r, r, zFloor) && np.z < zFloor + r) { np.z = zFloor + r; nv.z = 0.0f; return true; }
        return false;
    }
    bool settleOnFloor(F3& np, F3& nv, float zFrom, float r) const {
        float zFloor;
        if (floorUnderReach(np, zFrom, P.floor_settle_reach, r, zFloor)) { np.z = zFloor + r; nv.z = 0.0f; return true; }
        return false;
    }
    // clearWalls, the analytic venue's branch (cpu_crowd_sim.cpp:386-399): clearance r from the wall query
    bool clearWalls(F3& np, F3& nv, F3& wall, float r) const {
        bool moved = false;
        wall = {0.0f, 0.0f, 0.0f};
        for (int pass = 0; pass < P.wall_passes; ++pass) {
            const F3 w = this->wall(xy(np), P.feeler_reach);
            if (w.z >= r) {
                if (w.z < WALL_NONE) wall = {w.x, w.y, w.z - r};
                break;
            }
            setXY(np, xy(np) + F2{w.x, w.y} * (r - w.z));
            moved = true;
            wall = {w.x, w.y, 0.0f};
            const float vDotN = dot(xy(nv), F2{w.x, w.y});
            if (vDotN < 0.0f) setXY(nv, xy(nv) - F2{w.x, w.y} * vDotN);
        }
        return moved;
    }
    // wallPlaneProbe, the analytic venue's branch (cpu_crowd_sim.cpp:444-447)
    F3 wallPlaneProbe(F3 np, float r) const {
        const F3 w = wall(xy(np), P.plane_probe_reach);
        return w.z >= 0.0f && w.z < WALL_NONE ? F3{w.x, w.y, std::max(w.z - r, 0.0f)} : F3{0.0f, 0.0f, 0.0f};
    }
    bool solid(F3 p) const { return map(p) <= 0.0f; }
    // sweepBack (cpu_crowd_sim.cpp:465-479) over the grid's solid
    bool sweepBack(F3 pOld, F3& np, F3& nv) const {
        if (!solid(np)) return false;
        float lo = 0.0f, hi = 1.0f;
        if (!solid(F3{np.x, np.y, pOld.z})) lo = 1.0f;
        for (int i = 0; i < P.sweep_bisections; ++i) {
            float t = 0.5f * (lo + hi);
            F2 m = mix(xy(pOld), xy(np), t);
            if (solid(F3{m.x, m.y, pOld.z})) hi = t;
            else lo = t;
        }
        F2 d = safeNormalize(xy(np) - xy(pOld), P.safe_eps);
        F2 m = mix(xy(pOld), xy(np), lo);
        np = {m.x, m.y, pOld.z};
        float vd = dot(xy(nv), d);
        if (vd > 0.0f) setXY(nv, xy(nv) - d * vd);
        nv.z = 0.0f;
        return true;
    }
    // resolveStatic (cpu_crowd_sim.cpp:483-514) without the fence
    bool resolveStatic(F3 pOld, F3& np, F3& nv, bool settle, F3& wall, uint8_t& contact, float r) const {
        bool grounded = settle ? settleOnFloor(np, nv, pOld.z, r) : restOnFloor(np, nv, pOld.z, r);
        if (!grounded && sweepBack(pOld, np, nv)) {
            contact |= C_SWEEP;
            grounded = restOnFloor(np, nv, pOld.z, r);
        }
        if (grounded) contact |= C_FLOOR;
        const bool walls = clearWalls(np, nv, wall, r);
        if (walls) {
            contact |= C_WALL;
            if (grounded) {
                if (settleOnFloor(np, nv, pOld.z, r)) contact |= C_FLOOR;
                F3 w2;
                const bool again = clearWalls(np, nv, w2, r);
                if (w2.x != 0.0f || w2.y != 0.0f) wall = w2;
                if (again && restOnFloor(np, nv, pOld.z, r)) contact |= C_FLOOR;
            } else if (restOnFloor(np, nv, pOld.z, r)) {
                contact |= C_FLOOR;
            }
        }
        return grounded;
    }
    // The step-up limit over the floor heightfield (cpu_crowd_sim.cpp:566-591 limitStepUp, baked branch, with the
    // floor grid in place of the baked column scan). The nearest-node floor is level treads with vertical risers, the
    // reference's "exact venue": a floor in the window (f0 + tol, f0 + max] is never wall-steep, so only rule (a)
    // blocks (stepUpBlocked :531-533): the floor under the move's end more than max_step_up above f0. No floor grid:
    // flat, never blocked.
    int stepUpWindow(F2 p, float f0) const {   // 0 level or lower, 1 in the window, 2 above it
        const float h = floorHeight(p);
        if (h > f0 + P.max_step_up) return 2;
        return h > f0 + P.step_up_tol ? 1 : 0;
    }
    // the riser's normal: central differences of the floor over the neighbouring nodes, out of the higher column
    F2 stepUpFace(F2 p) const {
        const float fx = (p.x - V.wall_origin_x) * wallInvH + 0.5f, fy = (p.y - V.wall_origin_y) * wallInvH + 0.5f;
        const int ix = std::clamp(int(std::floor(fx)), 0, V.wall_nx - 1), iy = std::clamp(int(std::floor(fy)), 0, V.wall_ny - 1);
        const int x0 = std::max(ix - 1, 0), x1 = std::min(ix + 1, V.wall_nx - 1);
        const int y0 = std::max(iy - 1, 0), y1 = std::min(iy + 1, V.wall_ny - 1);
        const size_t row = size_t(iy) * size_t(V.wall_nx);
        const float* H = V.floor_height;
        const F2 g{H[row + size_t(x0)] - H[row + size_t(x1)],
                   H[size_t(y0) * size_t(V.wall_nx) + size_t(ix)] - H[size_t(y1) * size_t(V.wall_nx) + size_t(ix)]};
        return safeNormalize(g, P.safe_eps);
    }
    // cpu_crowd_sim.cpp:539-563 stepUpScan: only the end can block; the last allowed sample starts the bisection
    float stepUpScan(F2 p0, F2 p1, float f0, F2& n) const {
        n = {0.0f, 0.0f};
        const float len = length(p1 - p0);
        const int ns = std::clamp(int(std::ceil(len / P.step_up_sample)), 1, P.step_up_max_samples);
        const F2 pe = mix(p0, p1, float(ns) / float(ns));
        if (stepUpWindow(pe, f0) != 2) return 1.0f;
        n = stepUpFace(pe);
        int lastOk = 0;
        for (int i = 1; i < ns; ++i)
            if (stepUpWindow(mix(p0, p1, float(i) / float(ns)), f0) != 2) lastOk = i;
        float lo = float(lastOk) / float(ns), hi = float(lastOk + 1) / float(ns);
        for (int i = 0; i < P.step_up_bisections; ++i) {
            const float t = 0.5f * (lo + hi);
            const F2 q = mix(p0, p1, t);
            if (stepUpWindow(q, f0) == 2) { hi = t; n = stepUpFace(q); }
            else lo = t;
        }
        return lo;
    }
    // cpu_crowd_sim.cpp:566-591 limitStepUp: back to the riser, the rest along it (veering by the slide angles until
    // one is allowed), the velocity into it removed, settled from the start-of-step height; radius r the agent's own
    bool limitStepUp(F3 pOld, F3& np, F3& nv, float r) const {
        if (!V.floor_height) return false;
        float f0;
        if (!floorUnderReach(pOld, pOld.z, P.step_up_floor_reach, r, f0)) f0 = pOld.z - P.step_up_floor_reach;
        F2 n;
        const float t = stepUpScan(xy(pOld), xy(np), f0, n);
        if (t >= 1.0f) return false;
        F2 q = mix(xy(pOld), xy(np), t);
        const F2 rest = xy(np) - q;
        const F2 tangent = rest - n * dot(rest, n);
        const float lt = length(tangent);
        if (lt > 0.0f) {
            for (int k = 0; k < P.step_up_slide_tries; ++k) {
                const F2 slide = q + tangent * P.step_up_slide[k][0] + n * (lt * P.step_up_slide[k][1]);
                F2 n2;
                if (stepUpScan(q, slide, f0, n2) >= 1.0f) { q = slide; break; }
            }
        }
        const float vn = dot(xy(nv), n);
        if (vn < 0.0f) setXY(nv, xy(nv) - n * vn);
        float zFloor;
        if (floorUnderReach(F3{q.x, q.y, pOld.z}, pOld.z, P.floor_settle_reach, r, zFloor)) {
            np = F3{q.x, q.y, zFloor + r};
            nv.z = 0.0f;
        } else {
            np = F3{q.x, q.y, std::min(np.z, pOld.z)};
        }
        return true;
    }
    F3 calcGradient(F3 p) const {   // cpu_crowd_sim.cpp:312-318 over the grid's map
        const F3 kxyy{1.0f, -1.0f, -1.0f}, kyyx{-1.0f, -1.0f, 1.0f}, kyxy{-1.0f, 1.0f, -1.0f}, kxxx{1.0f, 1.0f, 1.0f};
        const float h = P.obstacle_grad_h;
        F3 a = kxyy * map(p + kxyy * h), b = kyyx * map(p + kyyx * h), c = kyxy * map(p + kyxy * h), d = kxxx * map(p + kxxx * h);
        return (a + b + c + d) * P.obstacle_grad_scale;
    }
};

// ================================================================================================================
// The step
// ================================================================================================================
struct Sim {
    SwarmParams P;
    SwarmVenue V;
    std::vector<float> sdf, wallSdf, navDist, floorH, speedF, exitBoxes;
    std::vector<uint8_t> exitMask;
    int threads;
    int n = 0;
    std::vector<Boid> boids[2];
    int readIdx = 0, writeIdx = 1;
    std::vector<Pair> grid, gridScratch;
    std::vector<Cell> cells;
    std::vector<uint32_t> bucketStart;
    std::vector<Boid> slotA, slotB;
    std::vector<F4> planes;
    std::vector<uint8_t> contacts;
    std::vector<float> radius, v0;
    std::vector<F2> drive;
    bool hasDrive = false;
    int resX, resY;
    // queue-aware exit choice (nav::choiceStep, src/exit_choice.cpp:671-790, restated on the hash cells' candidate
    // table): off while choiceExits == 0
    int choiceExits = 0, choiceK = 0;
    uint32_t choiceStep = 0;
    std::vector<float> exitFields, cDist, invCap;
    std::vector<uint8_t> cExit;
    std::vector<uint32_t> assign, pendExit, pendBin, hist, threshold, queue, ahead;
    uint32_t choiceCounters[4] = {0, 0, 0, 0};
    void resetChoice() {
        choiceStep = 0;
        assign.assign(size_t(n), SWARM_CHOICE_NONE);
        pendExit.assign(size_t(n), SWARM_CHOICE_NONE);
        pendBin.assign(size_t(n), 0u);
        hist.assign(size_t(choiceExits) * CHOICE_GAIN_BINS, 0u);
        threshold.assign(CHOICE_STRIDE, 0u);
        queue.assign(2 * CHOICE_STRIDE, 0u);
        ahead.assign(size_t(2) * CHOICE_STRIDE * CHOICE_AHEAD_BINS, 0u);
        for (auto& c : choiceCounters) c = 0;
    }
    void choicePass();

    Sim(const SwarmParams& p, const SwarmVenue& v, int nThreads) : P(p), V(v), threads(nThreads > 0 ? nThreads : omp_get_max_threads()) {
        resX = V.grid_res_x; resY = V.grid_res_y;
        if (V.kind == SWARM_VENUE_STADIUM) {
            size_t nv = size_t(V.sdf_res) * size_t(V.sdf_res) * size_t(V.sdf_res);
            sdf.assign(V.sdf, V.sdf + nv);
            V.sdf = sdf.data();
        } else {
            wallSdf.assign(V.wall_sdf, V.wall_sdf + size_t(V.wall_nx) * size_t(V.wall_ny));
            V.wall_sdf = wallSdf.data();
            navDist.assign(V.nav_dist, V.nav_dist + size_t(V.nav_nx) * size_t(V.nav_ny));
            V.nav_dist = navDist.data();
            if (V.floor_height) { floorH.assign(V.floor_height, V.floor_height + wallSdf.size()); V.floor_height = floorH.data(); }
            if (V.speed_factor) { speedF.assign(V.speed_factor, V.speed_factor + wallSdf.size()); V.speed_factor = speedF.data(); }
            if (V.exit_mask) { exitMask.assign(V.exit_mask, V.exit_mask + navDist.size()); V.exit_mask = exitMask.data(); }
        }
        if (V.n_exits > 0 && V.exit_boxes) { exitBoxes.assign(V.exit_boxes, V.exit_boxes + 4 * V.n_exits); V.exit_boxes = exitBoxes.data(); }
        cells.assign(size_t(resX) * size_t(resY), Cell{0, 0});
        bucketStart.assign(size_t(resX) * size_t(resY) + 2, 0);
    }

    void setState(const float* b, int count) {
        n = count;
        boids[0].resize(size_t(n));
        std::memcpy(boids[0].data(), b, size_t(n) * sizeof(Boid));
        boids[1] = boids[0];
        grid.assign(size_t(n), Pair{0, 0});
        gridScratch.assign(size_t(n), Pair{0, 0});
        slotA.assign(size_t(n), Boid{});
        slotB.assign(size_t(n), Boid{});
        planes.assign(size_t(n), F4{0, 0, 0, 0});
        contacts.assign(size_t(n), 0);
        if (radius.size() != size_t(n)) { radius.assign(size_t(n), P.body_radius); v0.assign(size_t(n), P.v_max); }
        resetChoice();
    }

    // cpu_crowd_sim.cpp:82-86 cellID, generalised to a rectangular grid
    uint32_t cellID(F2 p) const {
        int x = std::clamp(int((p.x - V.domain_min_x) / V.domain_span_x * float(resX)), 0, resX - 1);
        int y = std::clamp(int((p.y - V.domain_min_y) / V.domain_span_y * float(resY)), 0, resY - 1);
        return uint32_t(x + y * resX);
    }

    // cpu_crowd_sim.cpp:983-993 hash (with the NaN sanitiser of calc_grid.comp:24)
    void hash() {
        Boid* b = boids[readIdx].data();
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int id = 0; id < n; ++id) {
            if (std::isnan(b[id].pos.x)) b[id].pos = F4{0.0f, 0.0f, 0.0f, 1.0f};
            const F4 p = b[id].pos;
            grid[size_t(id)] = Pair{p.w == 0.0f ? INACTIVE_CELL : cellID(xy(p)), uint32_t(id)};
        }
    }
    // cpu_crowd_sim.cpp:997-1006 sortCounting: stable by cell, inactive bucket last
    void sortCounting() {
        const uint32_t inactive = uint32_t(resX * resY);
        auto bucketOf = [inactive](uint32_t g) { return g == INACTIVE_CELL ? inactive : g; };
        std::fill(bucketStart.begin(), bucketStart.end(), 0u);
        for (int i = 0; i < n; ++i) ++bucketStart[bucketOf(grid[size_t(i)].key) + 1];
        for (size_t k = 1; k < bucketStart.size(); ++k) bucketStart[k] += bucketStart[k - 1];
        for (int i = 0; i < n; ++i) gridScratch[bucketStart[bucketOf(grid[size_t(i)].key)]++] = grid[size_t(i)];
        std::swap(grid, gridScratch);
    }
    // cpu_crowd_sim.cpp:1034-1043 buildCells
    void buildCells() {
        std::fill(cells.begin(), cells.end(), Cell{0, 0});
        for (int id = 0; id < n; ++id) {
            const uint32_t g = grid[size_t(id)].key;
            if (g == INACTIVE_CELL) continue;
            ++cells[g].count;
            if (id == 0 || g != grid[size_t(id - 1)].key) cells[g].start = uint32_t(id);
        }
    }

    template <class Venue> void physics(const Venue& ven);
    void step() {
        if (choiceExits) choicePass();
        hash();
        sortCounting();
        buildCells();
        if (V.kind == SWARM_VENUE_STADIUM) {
            Stadium s{P, V.sdf, V.sdf_res, F3{V.sdf_origin[0], V.sdf_origin[1], V.sdf_origin[2]}, V.sdf_spacing, 1.0f / V.sdf_spacing,
                      F2{P.fence_center[0], P.fence_center[1]}, F2{P.fence_half_mid[0], P.fence_half_mid[1]},
                      V.domain_min_x, V.domain_span_x, V.domain_min_x + V.domain_span_x, V.exit_hi_x, V.exit_max_z, resX};
            physics(s);
        } else {
            GridVenue g{P, V, 1.0f / V.wall_h, 1.0f / V.nav_h, V.domain_min_x, V.domain_min_y,
                        V.domain_min_x + V.domain_span_x, V.domain_min_y + V.domain_span_y};
            physics(g);
        }
        std::swap(readIdx, writeIdx);
    }
};

// nav::choiceStep (src/exit_choice.cpp:671-790): the prefix stage, evaluate and thresholds on evaluation steps, apply;
// sequential in agent order (every count an integer: the GPU's atomics give the same)
void Sim::choicePass() {
    const uint32_t par = choiceStep & 1u;
    uint32_t* aRead = ahead.data() + size_t(par) * CHOICE_STRIDE * CHOICE_AHEAD_BINS;
    uint32_t* aWrite = ahead.data() + size_t(1u - par) * CHOICE_STRIDE * CHOICE_AHEAD_BINS;
    const int steps = std::max(1, int(CHOICE_T_S / double(P.dt) + 0.5));
    const bool evalStep = choiceStep > 0u && choiceStep % uint32_t(steps) == 0u;
    const int K = choiceK;
    for (int e = 0; e < choiceExits; ++e) {
        uint32_t run = 0;
        for (int b = 0; b < CHOICE_AHEAD_BINS; ++b) {
            const size_t i = size_t(e) * CHOICE_AHEAD_BINS + size_t(b);
            const uint32_t h = aRead[i];
            aRead[i] = run;
            run += h;
            aWrite[i] = 0u;
        }
    }
    for (int e = 0; e < CHOICE_STRIDE; ++e) queue[(1u - par) * CHOICE_STRIDE + uint32_t(e)] = 0u;
    auto bin = [](float d) { return std::min(uint32_t(d * 2.0f), uint32_t(CHOICE_AHEAD_BINS - 1)); };
    auto est = [&](float d, uint32_t e, uint32_t q) {
        const float walk = d * CHOICE_S_PER_M;
        const float wait = float(q) * invCap[e];
        return walk + wait;
    };
    auto slotOf = [&](size_t row, uint32_t e) {
        int k = -1;
        for (int i = 0; i < K; ++i) if (uint32_t(cExit[row + size_t(i)]) == e) k = i;
        return k;
    };
    auto bestOf = [&](size_t row, float& eBest) {
        int best = -1;
        eBest = 0.0f;
        for (int k = 0; k < K; ++k) {
            const uint32_t ex = cExit[row + size_t(k)];
            if (ex == SWARM_CHOICE_EMPTY) break;
            const float d = cDist[row + size_t(k)];
            const float e = est(d, ex, aRead[size_t(ex) * CHOICE_AHEAD_BINS + bin(d)]);
            if (best < 0 || e < eBest) { best = k; eBest = e; }
        }
        return best;
    };
    auto rowOf = [&](int i, size_t& row) {
        F4 p = boids[readIdx][size_t(i)].pos;
        if (std::isnan(p.x)) p = F4{0.0f, 0.0f, 0.0f, 1.0f};
        if (p.w == 0.0f) return false;
        row = size_t(cellID(xy(p))) * size_t(K);
        return true;
    };
    if (evalStep) {
        for (int i = 0; i < n; ++i) {
            pendExit[size_t(i)] = SWARM_CHOICE_NONE;
            pendBin[size_t(i)] = 0u;
            size_t row;
            if (!rowOf(i, row) || cExit[row] == SWARM_CHOICE_EMPTY) continue;
            const uint32_t cur = assign[size_t(i)];
            const int curK = slotOf(row, cur);
            if (curK < 0) continue;
            ++choiceCounters[0];
            float eBest;
            const int best = bestOf(row, eBest);
            const float dCur = cDist[row + size_t(curK)];
            const float eCur = est(dCur, cur, aRead[size_t(cur) * CHOICE_AHEAD_BINS + bin(dCur)]);
            const float gain = eCur - eBest;
            if (best != curK && gain > std::max(CHOICE_REL_MARGIN * eCur, CHOICE_ABS_MARGIN_S)) {
                const uint32_t b = std::min(uint32_t(gain), uint32_t(CHOICE_GAIN_BINS - 1));
                pendExit[size_t(i)] = cExit[row + size_t(best)];
                pendBin[size_t(i)] = b;
                ++hist[size_t(cur) * CHOICE_GAIN_BINS + b];
                ++choiceCounters[1];
            }
        }
        for (int e = 0; e < choiceExits; ++e) {   // nav::switchThreshold (src/exit_choice.cpp:625-640)
            uint32_t* h = hist.data() + size_t(e) * CHOICE_GAIN_BINS;
            const uint32_t queued = queue[par * CHOICE_STRIDE + uint32_t(e)];
            const uint32_t cap = std::max(CHOICE_MIN_SWITCHES, uint32_t(float(queued) * CHOICE_SWITCH_SHARE));
            uint32_t cum = 0, thr = uint32_t(CHOICE_GAIN_BINS);
            for (int b = CHOICE_GAIN_BINS - 1; b >= 0; --b) {
                const uint32_t c = h[b];
                if (c == 0) continue;
                if (cum + c > cap) {
                    if (cum == 0) thr = uint32_t(b);
                    break;
                }
                cum += c;
                thr = uint32_t(b);
            }
            threshold[size_t(e)] = thr;
            std::fill(h, h + CHOICE_GAIN_BINS, 0u);
        }
    }
    for (int i = 0; i < n; ++i) {   // nav::apply (src/exit_choice.cpp:642-658) and the counts for the next step
        size_t row;
        if (!rowOf(i, row)) continue;
        const uint32_t cur = assign[size_t(i)];
        uint32_t ex = cur;
        const bool hasPath = cExit[row] != SWARM_CHOICE_EMPTY;
        const int curK = hasPath ? slotOf(row, cur) : -1;
        if (hasPath && curK < 0) {
            float eBest;
            ex = cExit[row + size_t(bestOf(row, eBest))];
            if (cur != SWARM_CHOICE_NONE) ++choiceCounters[3];
        } else if (evalStep && curK >= 0 && pendExit[size_t(i)] != SWARM_CHOICE_NONE && pendBin[size_t(i)] >= threshold[cur]) {
            ex = pendExit[size_t(i)];
            ++choiceCounters[2];
        }
        assign[size_t(i)] = ex;
        if (ex != SWARM_CHOICE_NONE) {
            ++queue[(1u - par) * CHOICE_STRIDE + ex];
            const int k = slotOf(row, ex);
            if (k >= 0) ++aWrite[size_t(ex) * CHOICE_AHEAD_BINS + bin(cDist[row + size_t(k)])];
        }
    }
    ++choiceStep;
}

// The per-venue hooks the skeleton calls
inline bool venueExits(const Stadium& s, F4 p) { return s.exits(p); }
inline bool venueExits(const GridVenue& g, F4 p) { return g.exits(p); }
inline F2 venueGoal(const Stadium& s, F3 p) { return s.goal(p); }
inline F2 venueGoal(const GridVenue& g, F3 p) { return g.goal(p); }
inline F2 venueGoalIn(const Stadium& s, const float*, F3 p) { return s.goal(p); }
inline F2 venueGoalIn(const GridVenue& g, const float* D, F3 p) { return g.goalIn(D, p); }

template <class Venue>
struct Physics {
    const Sim& S;
    const SwarmParams& P;
    const Venue& ven;
    const Boid* boidsIn;
    Boid* boidsOut;
    const Boid* slotIn;
    Boid* slotOut;
    F4* planes;
    uint8_t* contacts;
    static constexpr bool kUniform = std::is_same<Venue, Stadium>::value;

    F2 goalDirection(F3 p, uint32_t id) const {   // cpu_crowd_sim.cpp:213-218
        if (S.hasDrive) return S.drive[id];
        if (S.choiceExits && S.assign[id] != SWARM_CHOICE_NONE)   // the assigned exit's own field
            return venueGoalIn(ven, S.exitFields.data() + size_t(S.assign[id]) * size_t(S.V.nav_nx) * size_t(S.V.nav_ny), p);
        return venueGoal(ven, p);
    }

    // cpu_crowd_sim.cpp:655-777 predict
    void predict(uint32_t slot) const {
        const uint32_t self = S.grid[slot].id, cid = S.grid[slot].key;
        uint8_t& contact = contacts[self];
        contact = 0;
        if (cid == INACTIVE_CELL) return;
        const F4 p = boidsIn[self].pos, v = boidsIn[self].vel;
        if (venueExits(ven, p)) {
            slotOut[slot].pos = F4{P.park_coord, P.park_coord, P.park_coord, 0.0f};
            slotOut[slot].vel = F4{0.0f, 0.0f, 0.0f, 0.0f};
            contact = C_EXIT;
            return;
        }
        const F2 eGoal = goalDirection(xyz(p), self);
        const float ri = kUniform ? P.body_radius : S.radius[self];
        const int cx = int(cid % uint32_t(S.resX)), cy = int(cid / uint32_t(S.resX));
        F2 sep{0.0f, 0.0f};
        float sAhead = 1e9f;   // uniform: the distance to the nearest agent ahead; per-agent: the smallest gap
        const int R = P.perc_ring;
        for (int y = -R; y <= R; y++) {
            for (int x = -R; x <= R; x++) {
                const int nx = cx + x, ny = cy + y;
                if (nx < 0 || nx >= S.resX || ny < 0 || ny >= S.resY) continue;
                const Cell cell = S.cells[size_t(nx + ny * S.resX)];
                for (uint32_t k = cell.start; k < cell.start + cell.count; k++) {
                    if (k == slot) continue;
                    const uint32_t other = S.grid[k].id;
                    const F4 op = boidsIn[other].pos;
                    const F3 offset = xyz(p) - xyz(op);
                    const float dxy2 = dot(xy(offset), xy(offset));
                    if (dxy2 < P.r_perc2) {
                        float dc, rs, rs2;
                        if (kUniform) { dc = P.body_diam; rs = P.r_sep; rs2 = P.r_sep2; }
                        else { dc = ri + S.radius[other]; rs = dc + P.sep_margin; rs2 = rs * rs; }
                        sep = sep + separationForce(P, offset, self, other, rs, rs2);
                        const float ahead = -dot(xy(offset), eGoal);
                        const float lateral = std::abs(offset.x * eGoal.y - offset.y * eGoal.x);
                        const float dxy = std::sqrt(dxy2);
                        const float key = kUniform ? dxy : dxy - dc;
                        if (ahead > 0.0f && lateral < dc && key < sAhead) {
                            const F2 eOther = goalDirection(xyz(op), other);
                            const float aheadOther = dot(xy(offset), eOther);
                            const bool mutual = aheadOther > 0.0f && std::abs(offset.x * eOther.y - offset.y * eOther.x) < dc;
                            if (!mutual || ahead > aheadOther || (ahead == aheadOther && self > other)) sAhead = key;
                        }
                    }
                }
            }
        }
        float vFree, vDes;
        if (kUniform) {
            vFree = P.v_max;
            vDes = std::clamp((sAhead - P.body_diam) * P.headway_rate, 0.0f, vFree) * length(eGoal);
        } else {
            vFree = S.v0[self] * venueSpeedFactor(xyz(p));
            vDes = std::clamp(sAhead * P.headway_rate, 0.0f, vFree) * length(eGoal);
        }
        const F2 eDir = safeNormalize(eGoal + sep, P.safe_eps);

        // obstacle avoidance at torso height (cpu_crowd_sim.cpp:737-747)
        F2 aObs{0.0f, 0.0f};
        const F3 torso{p.x, p.y, p.z + P.torso_height};
        bool onFence = false;
        const float dTorso = sceneDist(torso, onFence);
        if (dTorso < P.obstacle_range) {
            const F2 norm = sceneNormal(torso, onFence);
            if (length(norm) > P.obstacle_min_normal)
                aObs = safeNormalize(norm, P.safe_eps) * (P.obstacle_range - dTorso) * P.w_obs * P.obstacle_gain;
        }

        // kinematics (cpu_crowd_sim.cpp:751-766)
        const F2 vEq = eDir * vDes + aObs * P.tau_relax;
        F3 nv = xyz(v);
        setXY(nv, vEq + (xy(nv) - vEq) * P.relax_step);
        const float along = dot(xy(nv), eGoal);
        if (along > vDes) setXY(nv, xy(nv) - eGoal * (along - vDes));
        nv.z -= P.gravity_dt;
        nv.z = std::min(nv.z, 0.0f);
        if (length(xy(nv)) > P.v_max) setXY(nv, safeNormalize(xy(nv), P.safe_eps) * P.v_max);
        F3 np = xyz(p) + nv * P.dt;

        // static contacts, wall plane and grounded flag (cpu_crowd_sim.cpp:768-776)
        F3 wall;
        const bool grounded = resolveStatic(xyz(p), np, nv, false, wall, contact, ri);
        if (wall.x == 0.0f && wall.y == 0.0f) wall = wallPlaneProbe(np, ri);
        slotOut[slot].pos = F4{np.x, np.y, np.z, 1.0f};
        slotOut[slot].vel = F4{nv.x, nv.y, nv.z, 0.0f};
        const F2 wn{wall.x, wall.y};
        planes[slot] = F4{wn.x, wn.y, dot(xy(np), wn) - wall.z,
                          ((wn.x != 0.0f || wn.y != 0.0f) ? PLANE_WALL : 0.0f) + (grounded ? PLANE_GROUNDED : 0.0f)};
    }

    // venue dispatch
    float venueSpeedFactor(F3 p) const {
        if constexpr (kUniform) return 1.0f; else return ven.speedFactor(xy(p));
    }
    float sceneDist(F3 p, bool& onFence) const {
        if constexpr (kUniform) return ven.sceneDist(p, onFence);
        else { onFence = false; return ven.map(p); }
    }
    F2 sceneNormal(F3 p, bool onFence) const {
        if constexpr (kUniform) return ven.sceneNormal(p, onFence);
        else return xy(safeNormalize(ven.calcGradient(p), P.safe_eps));
    }
    bool resolveStatic(F3 pOld, F3& np, F3& nv, bool settle, F3& wall, uint8_t& contact, float r) const {
        if constexpr (kUniform) return ven.resolveStatic(pOld, np, nv, settle, wall, contact);
        else return ven.resolveStatic(pOld, np, nv, settle, wall, contact, r);
    }
    F3 wallPlaneProbe(F3 np, float r) const {
        if constexpr (kUniform) return ven.wallPlaneProbe(np);
        else return ven.wallPlaneProbe(np, r);
    }
    bool limitStepUp(F3 pOld, F3& np, F3& nv, float r) const {
        if constexpr (kUniform) return ven.limitStepUp(pOld, np, nv);
        else return ven.limitStepUp(pOld, np, nv, r);
    }

    // cpu_crowd_sim.cpp:781-822 projectSlot
    Boid projectSlot(uint32_t slot, uint32_t self, uint32_t cid) const {
        Boid b = slotIn[slot];
        if (b.pos.w == 0.0f) return b;
        const int cx = int(cid % uint32_t(S.resX)), cy = int(cid / uint32_t(S.resX));
        const float ri = kUniform ? P.body_radius : S.radius[self];
        F2 corr{0.0f, 0.0f};
        int nContacts = 0;
        for (int y = -1; y <= 1; y++) {
            for (int x = -1; x <= 1; x++) {
                const int nx = cx + x, ny = cy + y;
                if (nx < 0 || nx >= S.resX || ny < 0 || ny >= S.resY) continue;
                const Cell cell = S.cells[size_t(nx + ny * S.resX)];
                for (uint32_t k = cell.start; k < cell.start + cell.count; k++) {
                    if (k == slot) continue;
                    const F4 op = slotIn[k].pos;
                    const F3 offset = xyz(b.pos) - xyz(op);
                    float dc, dc2;
                    if (kUniform) { dc = P.body_diam; dc2 = P.body_diam2; }
                    else { dc = ri + S.radius[S.grid[k].id]; dc2 = dc * dc; }
                    if (op.w != 0.0f && std::abs(offset.z) < dc && dot(xy(offset), xy(offset)) < dc2) {
                        corr = corr + contactCorrection(P, offset, self, S.grid[k].id, dc, dc2);
                        ++nContacts;
                    }
                }
            }
        }
        corr = corr * (P.proj_relax / float(std::max(nContacts, 1)));
        const float len = length(corr);
        if (len > P.proj_max_shift) corr = corr * (P.proj_max_shift / len);
        F3 q = xyz(b.pos);
        setXY(q, xy(q) + corr);
        if constexpr (kUniform) ven.fenceProject(q);
        const F4 plane = planes[slot];
        if (std::fmod(plane.w, 2.0f) == PLANE_WALL) {
            const float s = plane.z - dot(xy(q), F2{plane.x, plane.y});
            if (s > 0.0f) setXY(q, xy(q) + F2{plane.x, plane.y} * s);
        }
        const F2 d = xy(q) - xy(b.pos);
        if (d != F2{0.0f, 0.0f}) contacts[self] |= C_AGENT;
        b.pos.x = q.x; b.pos.y = q.y;
        b.vel.w += length(d);
        return b;
    }

    void project(uint32_t slot) const {   // cpu_crowd_sim.cpp:825-831
        const uint32_t cid = S.grid[slot].key;
        if (cid != INACTIVE_CELL) slotOut[slot] = projectSlot(slot, S.grid[slot].id, cid);
    }

    // cpu_crowd_sim.cpp:835-866 finalPass
    void finalPass(uint32_t slot, bool projectHere) const {
        const uint32_t self = S.grid[slot].id, cid = S.grid[slot].key;
        if (cid == INACTIVE_CELL) { boidsOut[self] = boidsIn[self]; return; }
        const Boid b = projectHere ? projectSlot(slot, self, cid) : slotIn[slot];
        if (b.pos.w == 0.0f) { boidsOut[self] = b; return; }
        F3 np = xyz(b.pos), nv = xyz(b.vel);
        const F3 pOld = xyz(boidsIn[self].pos);
        const float ri = kUniform ? P.body_radius : S.radius[self];
        if (b.vel.w > 0.0f) {
            F3 wall;
            resolveStatic(pOld, np, nv, planes[slot].w >= PLANE_GROUNDED, wall, contacts[self], ri);
        }
        if (limitStepUp(pOld, np, nv, ri)) contacts[self] |= C_STEP_UP;
        boidsOut[self].pos = F4{np.x, np.y, np.z, 1.0f};
        boidsOut[self].vel = F4{nv.x, nv.y, nv.z, length(nv)};
    }
};

// cpu_crowd_sim.cpp:1055-1088 physics: predict -> slotA, K - 1 sweeps ping-ponging slotA / slotB, final pass
template <class Venue>
void Sim::physics(const Venue& ven) {
    Physics<Venue> ph{*this, P, ven, boids[readIdx].data(), boids[writeIdx].data(), nullptr, slotA.data(), planes.data(), contacts.data()};
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int s = 0; s < n; ++s) ph.predict(uint32_t(s));
    Boid* in = slotA.data();
    Boid* out = slotB.data();
    for (int it = 1; it < P.proj_iterations; ++it) {
        ph.slotIn = in;
        ph.slotOut = out;
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int s = 0; s < n; ++s) ph.project(uint32_t(s));
        std::swap(in, out);
    }
    ph.slotIn = in;
    ph.slotOut = nullptr;
    const bool projectInFinal = P.proj_iterations > 0;
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int s = 0; s < n; ++s) ph.finalPass(uint32_t(s), projectInFinal);
}

thread_local std::string g_err;

}  // namespace
}  // namespace oracle

using oracle::Sim;

extern "C" {

const char* oracle_last_error() { return oracle::g_err.c_str(); }

void* oracle_create(const SwarmParams* p, const SwarmVenue* v, int threads) {
    if (!p || !v) { oracle::g_err = "null argument"; return nullptr; }
    if (v->kind == SWARM_VENUE_STADIUM && !v->sdf) { oracle::g_err = "stadium venue without sdf"; return nullptr; }
    if (v->kind == SWARM_VENUE_GRID && (!v->wall_sdf || !v->nav_dist)) { oracle::g_err = "grid venue without fields"; return nullptr; }
    return new Sim(*p, *v, threads);
}
void oracle_destroy(void* h) { delete static_cast<Sim*>(h); }
int oracle_set_state(void* h, const float* boids, int n) {
    if (n <= 0) { oracle::g_err = "agent count out of range"; return -1; }
    static_cast<Sim*>(h)->setState(boids, n);
    return 0;
}
int oracle_set_agent_params(void* h, const float* radius, const float* v0, int n) {
    Sim* s = static_cast<Sim*>(h);
    s->radius.assign(radius, radius + n);
    s->v0.assign(v0, v0 + n);
    return 0;
}
int oracle_set_iterations(void* h, int k) {
    if (k < 0) { oracle::g_err = "iterations must be >= 0"; return -1; }
    static_cast<Sim*>(h)->P.proj_iterations = k;
    return 0;
}
int oracle_set_threads(void* h, int t) { Sim* s = static_cast<Sim*>(h); s->threads = t > 0 ? t : omp_get_max_threads(); return s->threads; }
int oracle_set_drive_table(void* h, const float* dirs, int n) {
    Sim* s = static_cast<Sim*>(h);
    if (!dirs) { s->hasDrive = false; s->drive.clear(); return 0; }
    s->drive.resize(size_t(n));
    std::memcpy(s->drive.data(), dirs, size_t(n) * 2 * sizeof(float));
    s->hasDrive = true;
    return 0;
}
// The queue-aware exit choice: the per-exit fields (n_exits x nav nodes), seconds per queued agent per exit, and the
// candidate table (ncells x K exits and distances, as swarm_exit_choice_table builds it); n_exits 0: off
int oracle_set_exit_choice(void* h, int nExits, int K, const float* fields, const float* invCap, const uint8_t* cExit,
                           const float* cDist) {
    Sim* s = static_cast<Sim*>(h);
    s->choiceExits = 0;
    if (nExits <= 0) { s->resetChoice(); return 0; }
    const size_t m = size_t(s->V.nav_nx) * size_t(s->V.nav_ny), rows = size_t(s->resX) * size_t(s->resY) * size_t(K);
    s->exitFields.assign(fields, fields + size_t(nExits) * m);
    s->invCap.assign(invCap, invCap + nExits);
    s->cExit.assign(cExit, cExit + rows);
    s->cDist.assign(cDist, cDist + rows);
    s->choiceExits = nExits;
    s->choiceK = K;
    s->resetChoice();
    return 0;
}
int oracle_get_exit_choice(void* h, uint32_t* assigned, uint32_t* counters) {
    Sim* s = static_cast<Sim*>(h);
    if (assigned) std::memcpy(assigned, s->assign.data(), size_t(s->n) * 4);
    if (counters) std::memcpy(counters, s->choiceCounters, 16);
    return 0;
}
int oracle_step(void* h, int steps) {
    Sim* s = static_cast<Sim*>(h);
    if (s->n == 0) { oracle::g_err = "no state"; return -1; }
    for (int i = 0; i < steps; ++i) s->step();
    return 0;
}
int oracle_get_state(void* h, float* out) {
    Sim* s = static_cast<Sim*>(h);
    std::memcpy(out, s->boids[s->readIdx].data(), size_t(s->n) * sizeof(oracle::Boid));
    return 0;
}
int oracle_get_grid(void* h, uint32_t* grid_id, uint32_t* boid_id) {
    Sim* s = static_cast<Sim*>(h);
    for (int i = 0; i < s->n; ++i) { grid_id[i] = s->grid[size_t(i)].key; boid_id[i] = s->grid[size_t(i)].id; }
    return 0;
}
int oracle_get_cells(void* h, uint32_t* start_count, int capacity) {
    Sim* s = static_cast<Sim*>(h);
    const int nc = int(s->cells.size());
    for (int i = 0; i < nc && i < capacity; ++i) { start_count[2 * i] = s->cells[size_t(i)].start; start_count[2 * i + 1] = s->cells[size_t(i)].count; }
    return nc;
}
int oracle_get_contacts(void* h, uint8_t* out) {
    Sim* s = static_cast<Sim*>(h);
    std::memcpy(out, s->contacts.data(), s->contacts.size());
    return 0;
}
int oracle_max_threads() { return omp_get_max_threads(); }

}  // extern "C"

// ================================================================================================================
// Safety metrics (src/metrics.cpp:249-268 cicDeposit / speedMass, :429-476 MetricsReference::record; the exit slot
// rule :40-51 for the stadium, exit boxes for grid venues)
// ================================================================================================================
namespace oracle {
namespace {
struct Metrics {
    SwarmParams P;
    SwarmVenue V;
    std::vector<float> boxes;
    int res;
    std::vector<uint32_t> thr;         // 4 per cell
    SwarmMetricCounters ctr{};
    std::vector<SwarmMetricCell> cells;
    std::vector<uint32_t> evac;
    uint32_t steps = 0;

    int exitSlot(F4 p) const {
        if (V.kind == SWARM_VENUE_STADIUM) {
            const float ax = std::abs(p.x), ay = std::abs(p.y);
            const bool alongY = ay >= ax;
            const float lat = alongY ? ax : ay;
            if (lat >= P.avenue_half) return 4;
            return alongY ? (p.y > 0.0f ? 2 : 3) : (p.x > 0.0f ? 0 : 1);
        }
        for (int e = 0; e < V.n_exits && e < 56; ++e) {
            const float* b = boxes.data() + 4 * e;
            if (p.x >= b[0] && p.x <= b[2] && p.y >= b[1] && p.y <= b[3]) return 5 + e;
        }
        return 4;
    }
    void record(const Boid* prev, const Boid* cur, int n) {
        ++steps;
        std::vector<uint32_t> mass(size_t(res) * size_t(res), 0u), smass(mass.size(), 0u);
        uint32_t active = 0;
        const float off = float(0.5 * res - 0.5);
        for (int i = 0; i < n; ++i) {
            const F4 p0 = prev[i].pos, p1 = cur[i].pos;
            if (p0.w != 0.0f && p1.w == 0.0f) {
                ++ctr.exits[exitSlot(p0)];
                ++ctr.evacuated;
                evac[size_t(i)] = steps;
            }
            if (p1.w != 0.0f) {
                ++active;
                const float gx = (p1.x - V.metric_center_x) * P.metric_cells_per_unit + off;
                const float gy = (p1.y - V.metric_center_y) * P.metric_cells_per_unit + off;
                const float fx = std::floor(gx), fy = std::floor(gy);
                const float tx = gx - fx, ty = gy - fy;
                const uint32_t qx = uint32_t(std::floor(tx * 256.0f + 0.5f)), qy = uint32_t(std::floor(ty * 256.0f + 0.5f));
                const uint32_t rx = 256u - qx, ry = 256u - qy;
                const int ix = int(fx), iy = int(fy);
                auto idx = [this](int x, int y) { return std::clamp(x, 0, res - 1) + std::clamp(y, 0, res - 1) * res; };
                const int c[4] = {idx(ix, iy), idx(ix + 1, iy), idx(ix, iy + 1), idx(ix + 1, iy + 1)};
                const uint32_t w[4] = {rx * ry, qx * ry, rx * qy, qx * qy};
                const float v = std::sqrt(cur[i].vel.x * cur[i].vel.x + cur[i].vel.y * cur[i].vel.y) * P.metric_speed_scale;
                for (int k = 0; k < 4; ++k) {
                    if (w[k] == 0) continue;
                    mass[size_t(c[k])] += w[k];
                    smass[size_t(c[k])] += uint32_t(std::floor(float(w[k]) * v + 0.5f));
                }
            }
        }
        ctr.active = active;
        ctr.active_accum = 0;
        ctr.step = steps;
        auto add64 = [](uint32_t* a, uint32_t b) {
            const uint64_t x = (uint64_t(a[0]) | (uint64_t(a[1]) << 32)) + b;
            a[0] = uint32_t(x); a[1] = uint32_t(x >> 32);
        };
        for (size_t c = 0; c < cells.size(); ++c) {
            const uint32_t m = mass[c], sm = smass[c];
            SwarmMetricCell& s = cells[c];
            s.last_mass = m;
            s.last_speed_mass = sm;
            s.peak_mass = std::max(s.peak_mass, m);
            s.occupied_steps += m != 0;
            for (int k = 0; k < 4; ++k) s.steps_above[k] += m >= thr[4 * c + size_t(k)];
            add64(s.mass_steps, m);
            add64(s.speed_mass_steps, sm);
            if (m >= thr[4 * c + 2]) add64(s.exposure_mass_steps, m);
        }
    }
};
}  // namespace
}  // namespace oracle

extern "C" {
void* oracle_metrics_create(const SwarmParams* p, const SwarmVenue* v, int res, const uint32_t* threshold_mass, int n) {
    auto* m = new oracle::Metrics{*p, *v, {}, res, {}, {}, {}, {}, 0};
    if (v->n_exits > 0 && v->exit_boxes) m->boxes.assign(v->exit_boxes, v->exit_boxes + 4 * v->n_exits);
    m->thr.assign(threshold_mass, threshold_mass + 4 * size_t(res) * size_t(res));
    m->cells.assign(size_t(res) * size_t(res), SwarmMetricCell{});
    m->evac.assign(size_t(n), 0u);
    return m;
}
void oracle_metrics_destroy(void* h) { delete static_cast<oracle::Metrics*>(h); }
int oracle_metrics_record(void* h, const float* prev, const float* cur, int n) {
    static_cast<oracle::Metrics*>(h)->record(reinterpret_cast<const oracle::Boid*>(prev), reinterpret_cast<const oracle::Boid*>(cur), n);
    return 0;
}
int oracle_metrics_read(void* h, SwarmMetricCounters* ctr, SwarmMetricCell* cells, uint32_t* evac) {
    auto* m = static_cast<oracle::Metrics*>(h);
    if (ctr) *ctr = m->ctr;
    if (cells) std::memcpy(cells, m->cells.data(), m->cells.size() * sizeof(SwarmMetricCell));
    if (evac) std::memcpy(evac, m->evac.data(), m->evac.size() * 4);
    return 0;
}
}
