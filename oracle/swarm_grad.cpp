// ORACLE -- test infrastructure only. Nothing in the product links, loads or calls this file: the gradient tests use
// it as the checker of the CUDA adjoint.
//
// Forward-mode derivatives of the grid-venue crowd step and of the evacuation loss
//
//     L = dt * sum_{t = 1..T} sum_{i active after step t} D(p_i(t)),
//
// D the bilinear interpolant of the venue's geodesic distance grid (the sample whose negative normalised gradient is
// e_goal). The step is the GRID branch of swarm_oracle.cpp (itself a restatement of DedovSergei/swarm-crowd-simulation
// src/cpu_crowd_sim.cpp: predict :655-777, projectSlot :781-822, finalPass :835-866, the analytic-venue static
// contacts :291-297, :386-399, :444-447, :465-514, the pair rules :127-152) written once over a scalar type S:
//
//   float              reproduces swarm_oracle.cpp bit for bit (tests/test_grad_oracle.py checks it)
//   double             the FP64 forward of the central finite differences
//   Dual<double, N>    exact directional derivatives of the FP64 forward, N directions per run
//   Dual<float, N>     directional derivatives along the FP32 trajectory: the primal arithmetic is the float
//                      instantiation's, operation for operation; the tangents are carried in double
//
// The derivatives are those of the branches the primal run takes: comparisons, clamps, the headway argmin and the
// contact activation read primal values only (the adjoint's frozen branch set). A branch signature, a hash of every
// discrete decision of the run, tells whether two runs (a finite-difference pair) took the same branches.
//
// The differentiated parameters: each agent's radius r_i and desired speed v0_i, and the relaxation time tau with
// relax_step = exp(-dt / tau) (the SI parameter set's definition).

#include "../include/swarm_cuda.h"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

namespace grad {
namespace {

constexpr uint32_t INACTIVE_CELL = 0xFFFFFFFFu;
constexpr float PLANE_WALL = 1.0f, PLANE_GROUNDED = 2.0f;
constexpr float WALL_NONE = 1e9f;

// ---- a forward-mode dual number: primal P, N tangents in double ----
template <class P, int N>
struct Dual {
    P v;
    double d[N];
    Dual() : v(P(0)) { for (double& x : d) x = 0.0; }
    Dual(P x) : v(x) { for (double& x2 : d) x2 = 0.0; }   // a constant
    friend Dual operator+(const Dual& a, const Dual& b) { Dual r; r.v = a.v + b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
    friend Dual operator-(const Dual& a, const Dual& b) { Dual r; r.v = a.v - b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
    friend Dual operator-(const Dual& a) { Dual r; r.v = -a.v; for (int i = 0; i < N; ++i) r.d[i] = -a.d[i]; return r; }
    friend Dual operator*(const Dual& a, const Dual& b) {
        Dual r;
        r.v = a.v * b.v;
        const double av = double(a.v), bv = double(b.v);
        for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * bv + av * b.d[i];
        return r;
    }
    friend Dual operator/(const Dual& a, const Dual& b) {
        Dual r;
        r.v = a.v / b.v;
        const double av = double(a.v), bv = double(b.v);
        for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] * bv - av * b.d[i]) / (bv * bv);
        return r;
    }
    friend bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
    friend bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
    friend bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
    friend bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
    friend bool operator==(const Dual& a, const Dual& b) { return a.v == b.v; }
    friend bool operator!=(const Dual& a, const Dual& b) { return a.v != b.v; }
    friend Dual sqrt(const Dual& a) {
        Dual r;
        r.v = std::sqrt(a.v);
        const double s = double(r.v);
        for (int i = 0; i < N; ++i) r.d[i] = s > 0.0 ? a.d[i] / (2.0 * s) : 0.0;
        return r;
    }
    friend Dual abs(const Dual& a) { return a.v < P(0) ? -a : a; }
};

template <class S> struct Prim { using type = S; };
template <class P, int N> struct Prim<Dual<P, N>> { using type = P; };
inline double val(float x) { return x; }
inline double val(double x) { return x; }
template <class P, int N> inline double val(const Dual<P, N>& x) { return double(x.v); }
template <class S> inline int ifloor(const S& x) {   // int(std::floor(x)) in the primal type
    using P = typename Prim<S>::type;
    return int(std::floor(P(val(x))));
}
template <class S> inline S cst(float x) { return S(typename Prim<S>::type(x)); }

// std::min / std::max / std::clamp exactly (the first argument wins ties)
template <class T> inline T smin(const T& a, const T& b) { return b < a ? b : a; }
template <class T> inline T smax(const T& a, const T& b) { return a < b ? b : a; }
template <class T> inline T sclamp(const T& v, const T& lo, const T& hi) { return v < lo ? lo : (hi < v ? hi : v); }

// ---- vectors in glm's operation order ----
template <class T> struct V2 { T x, y; };
template <class T> struct V3 { T x, y, z; };
template <class T> struct V4 { T x, y, z, w; };
template <class T> inline V2<T> operator+(V2<T> a, V2<T> b) { return {a.x + b.x, a.y + b.y}; }
template <class T> inline V2<T> operator-(V2<T> a, V2<T> b) { return {a.x - b.x, a.y - b.y}; }
template <class T> inline V2<T> operator-(V2<T> a) { return {-a.x, -a.y}; }
template <class T> inline V2<T> operator*(V2<T> a, T s) { return {a.x * s, a.y * s}; }
template <class T> inline V2<T> operator*(T s, V2<T> a) { return {s * a.x, s * a.y}; }
template <class T> inline V2<T> operator/(V2<T> a, T s) { return {a.x / s, a.y / s}; }
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> inline T dot(V2<T> a, V2<T> b) { return a.x * b.x + a.y * b.y; }
template <class T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline T length(V2<T> a) { using std::sqrt; return sqrt(dot(a, a)); }
template <class T> inline T length(V3<T> a) { using std::sqrt; return sqrt(dot(a, a)); }
template <class T> inline T mix(T a, T b, T t) { return a * (cst<T>(1.0f) - t) + b * t; }
template <class T> inline V2<T> mix(V2<T> a, V2<T> b, T t) { return {mix(a.x, b.x, t), mix(a.y, b.y, t)}; }
template <class T> inline V2<T> xy(V3<T> a) { return {a.x, a.y}; }
template <class T> inline V2<T> xy(V4<T> a) { return {a.x, a.y}; }
template <class T> inline V3<T> xyz(V4<T> a) { return {a.x, a.y, a.z}; }
template <class T> inline void setXY(V3<T>& v, V2<T> a) { v.x = a.x; v.y = a.y; }
template <class T> inline V2<T> safeNormalize(V2<T> v, T eps) {
    T l = length(v);
    return l > eps ? v / l : V2<T>{cst<T>(0.0f), cst<T>(0.0f)};
}
template <class T> inline V3<T> safeNormalize(V3<T> v, T eps) {
    T l = length(v);
    return l > eps ? V3<T>{v.x / l, v.y / l, v.z / l} : V3<T>{cst<T>(0.0f), cst<T>(0.0f), cst<T>(0.0f)};
}

inline uint32_t hash32(uint32_t x) {   // lowbias32 (cpu_crowd_sim.cpp:120-125)
    x ^= x >> 16; x *= 0x7feb352du;
    x ^= x >> 15; x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
template <class S> inline V2<S> pairDirection(uint32_t self, uint32_t other, float hashToRadians) {   // :127-133
    uint32_t lo = std::min(self, other), hi = std::max(self, other);
    float angle = float(hash32(hash32(lo) ^ hi)) * hashToRadians;
    V2<S> dir{cst<S>(std::cos(angle)), cst<S>(std::sin(angle))};
    return self == lo ? dir : -dir;
}

inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
// The branch signature of one agent in one step: its own decisions in order, its neighbour decisions as a set
struct Sig {
    uint64_t h = 1469598103934665603ull, set = 0;
    bool b(bool x) { h = (h ^ (x ? 0x9e37u : 0x79b9u)) * 1099511628211ull; return x; }
    void u(uint64_t x) { h = (h ^ mix64(x + 0x632be59bd9b4e019ull)) * 1099511628211ull; }
    void pair(uint32_t other, uint32_t flags) { set += mix64((uint64_t(other) << 8) ^ flags ^ 0x5851f42d4c957f2dull); }
    uint64_t value() const { return mix64(h ^ mix64(set)); }
};

// ---- the model constants in the scalar type; tau and relax_step carry the tau tangent ----
template <class S>
struct Prm {
    S dt, r_perc2, sep_margin, k_sep, headway_rate, tau_relax, relax_step, gravity_dt, proj_relax, proj_max_shift, safe_eps,
        stacked_xy2, torso_height, obstacle_range, w_obs, obstacle_gain, obstacle_min_normal, obstacle_grad_h,
        obstacle_grad_scale, feeler_reach, plane_probe_reach, floor_settle_reach, v_max, park_coord;
    float hash_to_radians;
    int perc_ring, wall_passes, sweep_bisections, K;
};

template <class S> inline S relaxOf(const S& tau, const SwarmParams& p);
template <> inline float relaxOf<float>(const float&, const SwarmParams& p) { return p.relax_step; }
template <> inline double relaxOf<double>(const double& tau, const SwarmParams& p) { return std::exp(-double(p.dt) / tau); }
template <class P, int N> struct RelaxDual {
    static Dual<P, N> get(const Dual<P, N>& tau, const SwarmParams& p) {
        Dual<P, N> r;
        const double t = double(tau.v), dt = double(p.dt);
        double rho;
        if constexpr (std::is_same<P, float>::value) { r.v = p.relax_step; rho = double(p.relax_step); }
        else { r.v = std::exp(-dt / t); rho = r.v; }
        for (int i = 0; i < N; ++i) r.d[i] = rho * dt / (t * t) * tau.d[i];   // d exp(-dt / tau) / d tau
        return r;
    }
};
template <class S> struct RelaxSel { static S get(const S& tau, const SwarmParams& p) { return relaxOf<S>(tau, p); } };
template <class P, int N> struct RelaxSel<Dual<P, N>> { static Dual<P, N> get(const Dual<P, N>& tau, const SwarmParams& p) { return RelaxDual<P, N>::get(tau, p); } };

template <class S>
Prm<S> makePrm(const SwarmParams& p, const S& tau) {
    Prm<S> q;
    q.dt = cst<S>(p.dt); q.r_perc2 = cst<S>(p.r_perc2); q.sep_margin = cst<S>(p.sep_margin); q.k_sep = cst<S>(p.k_sep);
    q.headway_rate = cst<S>(p.headway_rate); q.tau_relax = tau; q.relax_step = RelaxSel<S>::get(tau, p);
    q.gravity_dt = cst<S>(p.gravity_dt); q.proj_relax = cst<S>(p.proj_relax); q.proj_max_shift = cst<S>(p.proj_max_shift);
    q.safe_eps = cst<S>(p.safe_eps); q.stacked_xy2 = cst<S>(p.stacked_xy2); q.torso_height = cst<S>(p.torso_height);
    q.obstacle_range = cst<S>(p.obstacle_range); q.w_obs = cst<S>(p.w_obs); q.obstacle_gain = cst<S>(p.obstacle_gain);
    q.obstacle_min_normal = cst<S>(p.obstacle_min_normal); q.obstacle_grad_h = cst<S>(p.obstacle_grad_h);
    q.obstacle_grad_scale = cst<S>(p.obstacle_grad_scale); q.feeler_reach = cst<S>(p.feeler_reach);
    q.plane_probe_reach = cst<S>(p.plane_probe_reach); q.floor_settle_reach = cst<S>(p.floor_settle_reach);
    q.v_max = cst<S>(p.v_max); q.park_coord = cst<S>(p.park_coord);
    q.hash_to_radians = p.hash_to_radians;
    q.perc_ring = p.perc_ring; q.wall_passes = p.wall_passes; q.sweep_bisections = p.sweep_bisections; q.K = p.proj_iterations;
    return q;
}

// ---- the grid venue (swarm_oracle.cpp GridVenue over S) ----
template <class S>
struct GVen {
    const Prm<S>& P;
    const SwarmVenue& V;
    S wallInvH, navInvH;

    GVen(const Prm<S>& p, const SwarmVenue& v) : P(p), V(v), wallInvH(cst<S>(1.0f) / cst<S>(v.wall_h)), navInvH(cst<S>(1.0f) / cst<S>(v.nav_h)) {}

    V3<S> wall(V2<S> p, S reach, Sig& g) const {
        S fx = (p.x - cst<S>(V.wall_origin_x)) * wallInvH, fy = (p.y - cst<S>(V.wall_origin_y)) * wallInvH;
        if (g.b(!(fx >= cst<S>(0.0f) && fy >= cst<S>(0.0f) && fx <= cst<S>(float(V.wall_nx - 1)) && fy <= cst<S>(float(V.wall_ny - 1)))))
            return {cst<S>(0.0f), cst<S>(0.0f), cst<S>(WALL_NONE)};
        int ix = std::min(ifloor(fx), V.wall_nx - 2), iy = std::min(ifloor(fy), V.wall_ny - 2);
        g.u(uint64_t(ix) * 0x10001ull + uint64_t(iy));
        S wx = fx - cst<S>(float(ix)), wy = fy - cst<S>(float(iy));
        const float* W = V.wall_sdf;
        size_t r0 = size_t(iy) * size_t(V.wall_nx) + size_t(ix), r1 = r0 + size_t(V.wall_nx);
        S c00 = cst<S>(W[r0]), c10 = cst<S>(W[r0 + 1]), c01 = cst<S>(W[r1]), c11 = cst<S>(W[r1 + 1]);
        S d = mix(mix(c00, c10, wx), mix(c01, c11, wx), wy);
        if (g.b(d >= reach)) return {cst<S>(0.0f), cst<S>(0.0f), cst<S>(WALL_NONE)};
        V2<S> gr{mix(c10 - c00, c11 - c01, wy) * wallInvH, mix(c01 - c00, c11 - c10, wx) * wallInvH};
        V2<S> n = safeNormalize(gr, P.safe_eps);
        return {n.x, n.y, d};
    }
    S wallDist(V2<S> p, Sig& g) const { return wall(p, cst<S>(WALL_NONE), g).z; }
    size_t floorNode(V2<S> p) const {
        S fx = (p.x - cst<S>(V.wall_origin_x)) * wallInvH + cst<S>(0.5f), fy = (p.y - cst<S>(V.wall_origin_y)) * wallInvH + cst<S>(0.5f);
        int ix = std::clamp(ifloor(fx), 0, V.wall_nx - 1), iy = std::clamp(ifloor(fy), 0, V.wall_ny - 1);
        return size_t(iy) * size_t(V.wall_nx) + size_t(ix);
    }
    S floorHeight(V2<S> p) const { return V.floor_height ? cst<S>(V.floor_height[floorNode(p)]) : cst<S>(0.0f); }
    S speedFactor(V2<S> p) const { return V.speed_factor ? cst<S>(V.speed_factor[floorNode(p)]) : cst<S>(1.0f); }
    S map(V3<S> p, Sig& g) const {
        const S w = wallDist(xy(p), g), f = p.z - floorHeight(xy(p));
        g.b(f < w);
        return smin(w, f);
    }

    // the bilinear sample of the distance grid at p (clamped to the grid): value and e_goal
    void navSample(V2<S> p, S* dist, V2<S>* goal, Sig* g) const {
        S fx = (p.x - cst<S>(V.nav_origin_x)) * navInvH, fy = (p.y - cst<S>(V.nav_origin_y)) * navInvH;
        if (g) { g->b(fx < cst<S>(0.0f)); g->b(cst<S>(float(V.nav_nx - 1)) < fx); g->b(fy < cst<S>(0.0f)); g->b(cst<S>(float(V.nav_ny - 1)) < fy); }
        fx = sclamp(fx, cst<S>(0.0f), cst<S>(float(V.nav_nx - 1)));
        fy = sclamp(fy, cst<S>(0.0f), cst<S>(float(V.nav_ny - 1)));
        int ix = std::min(ifloor(fx), V.nav_nx - 2), iy = std::min(ifloor(fy), V.nav_ny - 2);
        if (g) g->u(uint64_t(ix) * 0x10001ull + uint64_t(iy) + 0x77ull);
        S wx = fx - cst<S>(float(ix)), wy = fy - cst<S>(float(iy));
        const float* D = V.nav_dist;
        size_t r0 = size_t(iy) * size_t(V.nav_nx) + size_t(ix), r1 = r0 + size_t(V.nav_nx);
        S d00 = cst<S>(D[r0]), d10 = cst<S>(D[r0 + 1]), d01 = cst<S>(D[r1]), d11 = cst<S>(D[r1 + 1]);
        if (dist) *dist = mix(mix(d00, d10, wx), mix(d01, d11, wx), wy);
        if (goal) {
            V2<S> gr{mix(d10 - d00, d11 - d01, wy), mix(d01 - d00, d11 - d10, wx)};
            *goal = safeNormalize(V2<S>{-gr.x, -gr.y}, P.safe_eps);
        }
    }
    V2<S> goal(V3<S> p, Sig* g) const { V2<S> e; navSample(xy(p), nullptr, &e, g); return e; }

    bool exits(V4<S> p) const {
        using Pt = typename Prim<S>::type;
        const double x = val(p.x), y = val(p.y), z = val(p.z);
        const float dmaxX = V.domain_min_x + V.domain_span_x, dmaxY = V.domain_min_y + V.domain_span_y;
        bool outDomain = x < V.domain_min_x || x > dmaxX || y < V.domain_min_y || y > dmaxY;
        if (V.exit_mask) {   // the exit mask: the nav node nearest to p (in the primal type)
            const Pt inv = Pt(1) / Pt(V.nav_h);
            const Pt fx = (Pt(x) - Pt(V.nav_origin_x)) * inv + Pt(0.5f), fy = (Pt(y) - Pt(V.nav_origin_y)) * inv + Pt(0.5f);
            const int ix = std::clamp(int(std::floor(fx)), 0, V.nav_nx - 1), iy = std::clamp(int(std::floor(fy)), 0, V.nav_ny - 1);
            return outDomain || V.exit_mask[size_t(iy) * size_t(V.nav_nx) + size_t(ix)] != 0;
        }
        bool out = x < V.exit_lo_x || x > V.exit_hi_x || y < V.exit_lo_y || y > V.exit_hi_y;
        return (out && z < V.exit_max_z) || outDomain;
    }

    bool floorUnderReach(V3<S> c, S zFrom, S down, S r, S& zFloor, Sig& g) const {
        const S h = floorHeight(xy(c));
        zFloor = h;
        if (g.b(c.z <= h)) return g.b(h <= smax(zFrom, c.z) + r);
        return g.b(h >= c.z - down);
    }
    bool restOnFloor(V3<S>& np, V3<S>& nv, S zFrom, S r, Sig& g) const {
        S zFloor;
        if (floorUnderReach(np, zFrom, r, r, zFloor, g) && g.b(np.z < zFloor + r)) { np.z = zFloor + r; nv.z = cst<S>(0.0f); return true; }
        return false;
    }
    bool settleOnFloor(V3<S>& np, V3<S>& nv, S zFrom, S r, Sig& g) const {
        S zFloor;
        if (floorUnderReach(np, zFrom, P.floor_settle_reach, r, zFloor, g)) { np.z = zFloor + r; nv.z = cst<S>(0.0f); return true; }
        return false;
    }
    bool clearWalls(V3<S>& np, V3<S>& nv, V3<S>& wl, S r, Sig& g) const {
        bool moved = false;
        wl = {cst<S>(0.0f), cst<S>(0.0f), cst<S>(0.0f)};
        for (int pass = 0; pass < P.wall_passes; ++pass) {
            const V3<S> w = this->wall(xy(np), P.feeler_reach, g);
            if (g.b(w.z >= r)) {
                if (g.b(w.z < cst<S>(WALL_NONE))) wl = {w.x, w.y, w.z - r};
                break;
            }
            setXY(np, xy(np) + V2<S>{w.x, w.y} * (r - w.z));
            moved = true;
            wl = {w.x, w.y, cst<S>(0.0f)};
            const S vDotN = dot(xy(nv), V2<S>{w.x, w.y});
            if (g.b(vDotN < cst<S>(0.0f))) setXY(nv, xy(nv) - V2<S>{w.x, w.y} * vDotN);
        }
        return moved;
    }
    V3<S> wallPlaneProbe(V3<S> np, S r, Sig& g) const {
        const V3<S> w = wall(xy(np), P.plane_probe_reach, g);
        if (g.b(w.z >= cst<S>(0.0f) && w.z < cst<S>(WALL_NONE))) {
            g.b(w.z - r < cst<S>(0.0f));
            return V3<S>{w.x, w.y, smax(w.z - r, cst<S>(0.0f))};
        }
        return V3<S>{cst<S>(0.0f), cst<S>(0.0f), cst<S>(0.0f)};
    }
    bool solid(V3<S> p, Sig& g) const { return g.b(map(p, g) <= cst<S>(0.0f)); }
    bool sweepBack(V3<S> pOld, V3<S>& np, V3<S>& nv, Sig& g) const {
        if (!solid(np, g)) return false;
        float lo = 0.0f, hi = 1.0f;
        if (!solid(V3<S>{np.x, np.y, pOld.z}, g)) lo = 1.0f;
        for (int i = 0; i < P.sweep_bisections; ++i) {
            float t = 0.5f * (lo + hi);
            V2<S> m = mix(xy(pOld), xy(np), cst<S>(t));
            if (solid(V3<S>{m.x, m.y, pOld.z}, g)) hi = t;
            else lo = t;
        }
        V2<S> d = safeNormalize(xy(np) - xy(pOld), P.safe_eps);
        V2<S> m = mix(xy(pOld), xy(np), cst<S>(lo));
        np = {m.x, m.y, pOld.z};
        S vd = dot(xy(nv), d);
        if (g.b(vd > cst<S>(0.0f))) setXY(nv, xy(nv) - d * vd);
        nv.z = cst<S>(0.0f);
        return true;
    }
    bool resolveStatic(V3<S> pOld, V3<S>& np, V3<S>& nv, bool settle, V3<S>& wl, S r, Sig& g) const {
        bool grounded = settle ? settleOnFloor(np, nv, pOld.z, r, g) : restOnFloor(np, nv, pOld.z, r, g);
        if (!grounded && sweepBack(pOld, np, nv, g)) grounded = restOnFloor(np, nv, pOld.z, r, g);
        const bool walls = clearWalls(np, nv, wl, r, g);
        if (walls) {
            if (grounded) {
                settleOnFloor(np, nv, pOld.z, r, g);
                V3<S> w2;
                const bool again = clearWalls(np, nv, w2, r, g);
                if (g.b(w2.x != cst<S>(0.0f) || w2.y != cst<S>(0.0f))) wl = w2;
                if (again) restOnFloor(np, nv, pOld.z, r, g);
            } else {
                restOnFloor(np, nv, pOld.z, r, g);
            }
        }
        return grounded;
    }
    V3<S> calcGradient(V3<S> p, Sig& g) const {   // cpu_crowd_sim.cpp:312-318 over the grid's map
        const S one = cst<S>(1.0f), m1 = cst<S>(-1.0f);
        const V3<S> kxyy{one, m1, m1}, kyyx{m1, m1, one}, kyxy{m1, one, m1}, kxxx{one, one, one};
        const S h = P.obstacle_grad_h;
        V3<S> a = kxyy * map(p + kxyy * h, g), b = kyyx * map(p + kyyx * h, g), c = kyxy * map(p + kyxy * h, g), d = kxxx * map(p + kxxx * h, g);
        return (a + b + c + d) * P.obstacle_grad_scale;
    }
};

// L accumulated in double (its tangents likewise) whatever the step's scalar
template <class S> struct Acc { using type = double; static double of(const S& x) { return double(x); } };
template <class P, int N> struct Acc<Dual<P, N>> {
    using type = Dual<double, N>;
    static Dual<double, N> of(const Dual<P, N>& x) { Dual<double, N> r(double(x.v)); for (int i = 0; i < N; ++i) r.d[i] = x.d[i]; return r; }
};

template <class S> struct Boid { V4<S> pos, vel; };
struct Pair { uint32_t key, id; };
struct Cell { uint32_t start, count; };

template <class S>
struct Run {
    const SwarmParams& SP;
    const SwarmVenue& V;
    Prm<S> P;
    GVen<S> ven;
    int n, resX, resY, threads;
    std::vector<S> radius, v0;
    std::vector<Boid<S>> boids[2];
    int readIdx = 0;
    std::vector<Pair> grid, scratch;
    std::vector<Cell> cells;
    std::vector<uint32_t> bucket;
    std::vector<Boid<S>> slotA, slotB;
    std::vector<V4<S>> planes;
    std::vector<Sig> sig;
    uint64_t signature = 0;

    Run(const SwarmParams& sp, const SwarmVenue& v, const S& tau, int count, int nThreads)
        : SP(sp), V(v), P(makePrm<S>(sp, tau)), ven(P, V), n(count), resX(v.grid_res_x), resY(v.grid_res_y), threads(nThreads) {
        for (auto& b : boids) b.resize(size_t(n));
        grid.resize(size_t(n)); scratch.resize(size_t(n));
        cells.resize(size_t(resX) * size_t(resY));
        bucket.resize(cells.size() + 2);
        slotA.resize(size_t(n)); slotB.resize(size_t(n)); planes.resize(size_t(n)); sig.resize(size_t(n));
    }

    uint32_t cellID(V2<S> p) const {   // cpu_crowd_sim.cpp:82-86 over a rectangular grid, in the primal type
        using Pt = typename Prim<S>::type;
        const Pt px = Pt(val(p.x)), py = Pt(val(p.y));
        int x = std::clamp(int((px - Pt(V.domain_min_x)) / Pt(V.domain_span_x) * Pt(resX)), 0, resX - 1);
        int y = std::clamp(int((py - Pt(V.domain_min_y)) / Pt(V.domain_span_y) * Pt(resY)), 0, resY - 1);
        return uint32_t(x + y * resX);
    }
    void sortAndCells() {   // hash :983-993, sortCounting :997-1006, buildCells :1034-1043
        Boid<S>* b = boids[readIdx].data();
        for (int id = 0; id < n; ++id) {
            if (std::isnan(val(b[id].pos.x))) b[id].pos = V4<S>{cst<S>(0.0f), cst<S>(0.0f), cst<S>(0.0f), cst<S>(1.0f)};
            grid[size_t(id)] = Pair{val(b[id].pos.w) == 0.0 ? INACTIVE_CELL : cellID(xy(b[id].pos)), uint32_t(id)};
        }
        const uint32_t inactive = uint32_t(resX * resY);
        auto bucketOf = [inactive](uint32_t g) { return g == INACTIVE_CELL ? inactive : g; };
        std::fill(bucket.begin(), bucket.end(), 0u);
        for (int i = 0; i < n; ++i) ++bucket[bucketOf(grid[size_t(i)].key) + 1];
        for (size_t k = 1; k < bucket.size(); ++k) bucket[k] += bucket[k - 1];
        for (int i = 0; i < n; ++i) scratch[bucket[bucketOf(grid[size_t(i)].key)]++] = grid[size_t(i)];
        std::swap(grid, scratch);
        std::fill(cells.begin(), cells.end(), Cell{0, 0});
        for (int id = 0; id < n; ++id) {
            const uint32_t g = grid[size_t(id)].key;
            if (g == INACTIVE_CELL) continue;
            ++cells[g].count;
            if (id == 0 || g != grid[size_t(id - 1)].key) cells[g].start = uint32_t(id);
        }
    }

    V2<S> separationForce(V3<S> offset, uint32_t self, uint32_t other, S rsep, S rsep2, Sig& g) const {   // :135-143
        using std::sqrt;
        S d2 = dot(offset, offset);
        if (d2 >= rsep2) return {cst<S>(0.0f), cst<S>(0.0f)};
        S w = cst<S>(1.0f) - sqrt(d2) / rsep;
        S magnitude = P.k_sep * w * w;
        S dxy2 = dot(xy(offset), xy(offset));
        if (g.b(dxy2 <= P.stacked_xy2)) return magnitude * pairDirection<S>(self, other, P.hash_to_radians);
        return magnitude * xy(offset) * (cst<S>(1.0f) / sqrt(dxy2));
    }
    V2<S> contactCorrection(V3<S> offset, uint32_t self, uint32_t other, S dc, S dc2, Sig& g) const {   // :145-152
        using std::abs; using std::sqrt;
        S dxy2 = dot(xy(offset), xy(offset));
        if (abs(offset.z) >= dc || dxy2 >= dc2) return {cst<S>(0.0f), cst<S>(0.0f)};
        S dxy = sqrt(dxy2);
        S shift = cst<S>(0.5f) * (dc - dxy);
        if (g.b(dxy2 <= P.stacked_xy2)) return shift * pairDirection<S>(self, other, P.hash_to_radians);
        return shift * (xy(offset) / dxy);
    }

    void predict(uint32_t slot) {   // cpu_crowd_sim.cpp:655-777, the GRID branch
        using std::abs; using std::sqrt;
        const Boid<S>* in = boids[readIdx].data();
        const uint32_t self = grid[slot].id, cid = grid[slot].key;
        Sig& g = sig[self];
        g = Sig{};
        if (cid == INACTIVE_CELL) return;
        const V4<S> p = in[self].pos, v = in[self].vel;
        if (g.b(ven.exits(p))) {
            slotA[slot].pos = V4<S>{P.park_coord, P.park_coord, P.park_coord, cst<S>(0.0f)};
            slotA[slot].vel = V4<S>{cst<S>(0.0f), cst<S>(0.0f), cst<S>(0.0f), cst<S>(0.0f)};
            return;
        }
        const V2<S> eGoal = ven.goal(xyz(p), &g);
        const S ri = radius[self];
        const int cx = int(cid % uint32_t(resX)), cy = int(cid / uint32_t(resX));
        V2<S> sep{cst<S>(0.0f), cst<S>(0.0f)};
        S sAhead = cst<S>(1e9f);
        uint32_t jstar = 0xFFFFFFFFu;
        const int R = P.perc_ring;
        for (int y = -R; y <= R; y++) {
            for (int x = -R; x <= R; x++) {
                const int nx = cx + x, ny = cy + y;
                if (nx < 0 || nx >= resX || ny < 0 || ny >= resY) continue;
                const Cell cell = cells[size_t(nx + ny * resX)];
                for (uint32_t k = cell.start; k < cell.start + cell.count; k++) {
                    if (k == slot) continue;
                    const uint32_t other = grid[k].id;
                    const V4<S> op = in[other].pos;
                    const V3<S> offset = xyz(p) - xyz(op);
                    const S dxy2 = dot(xy(offset), xy(offset));
                    if (dxy2 < P.r_perc2) {
                        const S dc = ri + radius[other];
                        const S rs = dc + P.sep_margin, rs2 = rs * rs;
                        uint32_t flags = dot(offset, offset) < rs2 ? 1u : 0u;
                        sep = sep + separationForce(offset, self, other, rs, rs2, g);
                        const S ahead = -dot(xy(offset), eGoal);
                        const S lateral = abs(offset.x * eGoal.y - offset.y * eGoal.x);
                        const S dxy = sqrt(dxy2);
                        const S key = dxy - dc;
                        if (ahead > cst<S>(0.0f) && lateral < dc) {
                            flags |= 2u;
                            if (key < sAhead) {
                                flags |= 4u;
                                const V2<S> eOther = ven.goal(xyz(op), nullptr);
                                const S aheadOther = dot(xy(offset), eOther);
                                const bool mutual = aheadOther > cst<S>(0.0f) && abs(offset.x * eOther.y - offset.y * eOther.x) < dc;
                                if (!mutual || ahead > aheadOther || (ahead == aheadOther && self > other)) { sAhead = key; jstar = other; }
                            }
                        }
                        g.pair(other, flags);
                    }
                }
            }
        }
        g.u(jstar);
        const S vFree = v0[self] * ven.speedFactor(xy(p));
        const S hw = sAhead * P.headway_rate;
        g.b(hw < cst<S>(0.0f)); g.b(vFree < hw);
        const S vDes = sclamp(hw, cst<S>(0.0f), vFree) * length(eGoal);
        const V2<S> eDir = safeNormalize(eGoal + sep, P.safe_eps);
        g.b(length(eGoal + sep) > P.safe_eps);

        V2<S> aObs{cst<S>(0.0f), cst<S>(0.0f)};
        const V3<S> torso{p.x, p.y, p.z + P.torso_height};
        const S dTorso = ven.map(torso, g);
        if (g.b(dTorso < P.obstacle_range)) {
            const V2<S> norm = xy(safeNormalize(ven.calcGradient(torso, g), P.safe_eps));
            if (g.b(length(norm) > P.obstacle_min_normal))
                aObs = safeNormalize(norm, P.safe_eps) * (P.obstacle_range - dTorso) * P.w_obs * P.obstacle_gain;
        }

        const V2<S> vEq = eDir * vDes + aObs * P.tau_relax;
        V3<S> nv = xyz(v);
        setXY(nv, vEq + (xy(nv) - vEq) * P.relax_step);
        const S along = dot(xy(nv), eGoal);
        if (g.b(along > vDes)) setXY(nv, xy(nv) - eGoal * (along - vDes));
        nv.z = nv.z - P.gravity_dt;
        g.b(cst<S>(0.0f) < nv.z);
        nv.z = smin(nv.z, cst<S>(0.0f));
        if (g.b(length(xy(nv)) > P.v_max)) setXY(nv, safeNormalize(xy(nv), P.safe_eps) * P.v_max);
        V3<S> np = xyz(p) + nv * P.dt;

        V3<S> wl;
        const bool grounded = ven.resolveStatic(xyz(p), np, nv, false, wl, ri, g);
        if (g.b(wl.x == cst<S>(0.0f) && wl.y == cst<S>(0.0f))) wl = ven.wallPlaneProbe(np, ri, g);
        slotA[slot].pos = V4<S>{np.x, np.y, np.z, cst<S>(1.0f)};
        slotA[slot].vel = V4<S>{nv.x, nv.y, nv.z, cst<S>(0.0f)};
        const V2<S> wn{wl.x, wl.y};
        const bool isWall = wn.x != cst<S>(0.0f) || wn.y != cst<S>(0.0f);
        planes[slot] = V4<S>{wn.x, wn.y, dot(xy(np), wn) - wl.z,
                             cst<S>((isWall ? PLANE_WALL : 0.0f) + (grounded ? PLANE_GROUNDED : 0.0f))};
    }

    Boid<S> projectSlot(uint32_t slot, const std::vector<Boid<S>>& slotIn) {   // cpu_crowd_sim.cpp:781-822
        Boid<S> b = slotIn[slot];
        if (val(b.pos.w) == 0.0) return b;
        const uint32_t self = grid[slot].id, cid = grid[slot].key;
        Sig& g = sig[self];
        const int cx = int(cid % uint32_t(resX)), cy = int(cid / uint32_t(resX));
        const S ri = radius[self];
        V2<S> corr{cst<S>(0.0f), cst<S>(0.0f)};
        int nContacts = 0;
        for (int y = -1; y <= 1; y++) {
            for (int x = -1; x <= 1; x++) {
                const int nx = cx + x, ny = cy + y;
                if (nx < 0 || nx >= resX || ny < 0 || ny >= resY) continue;
                const Cell cell = cells[size_t(nx + ny * resX)];
                for (uint32_t k = cell.start; k < cell.start + cell.count; k++) {
                    if (k == slot) continue;
                    const V4<S> op = slotIn[k].pos;
                    const V3<S> offset = xyz(b.pos) - xyz(op);
                    const S dc = ri + radius[grid[k].id], dc2 = dc * dc;
                    using std::abs;
                    if (val(op.w) != 0.0 && abs(offset.z) < dc && dot(xy(offset), xy(offset)) < dc2) {
                        corr = corr + contactCorrection(offset, self, grid[k].id, dc, dc2, g);
                        ++nContacts;
                        g.pair(grid[k].id, 0x100u + uint32_t(nContacts > 0));
                    }
                }
            }
        }
        g.u(uint64_t(nContacts) + 0x1000ull);
        using Pt = typename Prim<S>::type;
        corr = corr * (P.proj_relax / cst<S>(Pt(std::max(nContacts, 1))));
        const S len = length(corr);
        if (g.b(len > P.proj_max_shift)) corr = corr * (P.proj_max_shift / len);
        V3<S> q = xyz(b.pos);
        setXY(q, xy(q) + corr);
        const V4<S> plane = planes[slot];
        if (std::fmod(val(plane.w), 2.0) == double(PLANE_WALL)) {
            const S s = plane.z - dot(xy(q), V2<S>{plane.x, plane.y});
            if (g.b(s > cst<S>(0.0f))) setXY(q, xy(q) + V2<S>{plane.x, plane.y} * s);
        }
        const V2<S> d = xy(q) - xy(b.pos);
        b.pos.x = q.x; b.pos.y = q.y;
        b.vel.w = b.vel.w + length(d);
        return b;
    }

    void finalPass(uint32_t slot, const std::vector<Boid<S>>& slotIn, bool projectHere) {   // :835-866
        const Boid<S>* in = boids[readIdx].data();
        Boid<S>* out = boids[readIdx ^ 1].data();
        const uint32_t self = grid[slot].id, cid = grid[slot].key;
        if (cid == INACTIVE_CELL) { out[self] = in[self]; return; }
        const Boid<S> b = projectHere ? projectSlot(slot, slotIn) : slotIn[slot];
        if (val(b.pos.w) == 0.0) { out[self] = b; return; }
        Sig& g = sig[self];
        V3<S> np = xyz(b.pos), nv = xyz(b.vel);
        const V3<S> pOld = xyz(in[self].pos);
        const S ri = radius[self];
        if (g.b(b.vel.w > cst<S>(0.0f))) {
            V3<S> wl;
            ven.resolveStatic(pOld, np, nv, val(planes[slot].w) >= double(PLANE_GROUNDED), wl, ri, g);
        }
        out[self].pos = V4<S>{np.x, np.y, np.z, cst<S>(1.0f)};
        out[self].vel = V4<S>{nv.x, nv.y, nv.z, length(nv)};
    }

    // One step (cpu_crowd_sim.cpp:967-1088 for a grid venue); returns sum_i D(p_i) over the agents active after it,
    // summed in double in agent order
    typename Acc<S>::type step() {
        sortAndCells();
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int s = 0; s < n; ++s) predict(uint32_t(s));
        std::vector<Boid<S>>* in = &slotA;
        std::vector<Boid<S>>* out = &slotB;
        for (int it = 1; it < P.K; ++it) {
#pragma omp parallel for schedule(static) num_threads(threads)
            for (int s = 0; s < n; ++s) {
                if (grid[size_t(s)].key != INACTIVE_CELL) (*out)[size_t(s)] = projectSlot(uint32_t(s), *in);
            }
            std::swap(in, out);
        }
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int s = 0; s < n; ++s) finalPass(uint32_t(s), *in, P.K > 0);
        readIdx ^= 1;
        // the loss term and the step's signature, in agent order
        const Boid<S>* b = boids[readIdx].data();
        typename Acc<S>::type sum = typename Acc<S>::type(0.0);
        uint64_t h = 0;
        for (int i = 0; i < n; ++i) {
            if (val(b[i].pos.w) != 0.0) {
                S d;
                ven.navSample(xy(b[i].pos), &d, nullptr, nullptr);
                sum = sum + Acc<S>::of(d);
            }
            h = mix64(h ^ sig[size_t(i)].value() ^ (uint64_t(i) << 1));
        }
        signature = mix64(signature ^ h);
        return sum;
    }
};

// A parameter's tangent along directions 0 .. nt - 1: d[k * stride]
template <class S>
struct Seed {
    static void set(S&, const double*, int, int) {}
};
template <class P, int N>
struct Seed<Dual<P, N>> {
    static void set(Dual<P, N>& x, const double* d, int nt, int stride) { for (int k = 0; k < nt && k < N; ++k) x.d[k] = d[size_t(k) * size_t(stride)]; }
};

template <class S>
int runT(const SwarmParams& p, const SwarmVenue& v, const float* state, int n, const double* radius, const double* v0, double tau,
         int steps, int threads, int nt, const double* dr, const double* dv0, const double* dtau, double* loss, double* dloss,
         uint64_t* sig, float* stateOut) {
    using Pt = typename Prim<S>::type;
    S tauS = cst<S>(0.0f);
    tauS = S(Pt(tau));
    if (nt > 0 && dtau) Seed<S>::set(tauS, dtau, nt, 1);
    Run<S> R(p, v, tauS, n, threads);
    R.radius.resize(size_t(n));
    R.v0.resize(size_t(n));
    for (int i = 0; i < n; ++i) {
        R.radius[size_t(i)] = S(Pt(radius[i]));
        R.v0[size_t(i)] = S(Pt(v0[i]));
        if (nt > 0) {
            if (dr) Seed<S>::set(R.radius[size_t(i)], dr + i, nt, n);
            if (dv0) Seed<S>::set(R.v0[size_t(i)], dv0 + i, nt, n);
        }
        const float* b = state + size_t(i) * 8;
        R.boids[0][size_t(i)] = Boid<S>{{cst<S>(b[0]), cst<S>(b[1]), cst<S>(b[2]), cst<S>(b[3])}, {cst<S>(b[4]), cst<S>(b[5]), cst<S>(b[6]), cst<S>(b[7])}};
    }
    R.boids[1] = R.boids[0];
    using A = Acc<S>;
    typename A::type L = typename A::type(0.0);
    const typename A::type dt = typename A::type(double(p.dt));
    for (int t = 0; t < steps; ++t) L = L + dt * R.step();
    if constexpr (std::is_same<typename A::type, double>::value) {
        *loss = L;
    } else {
        *loss = L.v;
        if (dloss) for (int k = 0; k < nt; ++k) dloss[k] = L.d[k];
    }
    if (sig) *sig = R.signature;
    if (stateOut) {
        const auto& b = R.boids[R.readIdx];
        for (int i = 0; i < n; ++i) {
            float* o = stateOut + size_t(i) * 8;
            o[0] = float(val(b[size_t(i)].pos.x)); o[1] = float(val(b[size_t(i)].pos.y)); o[2] = float(val(b[size_t(i)].pos.z)); o[3] = float(val(b[size_t(i)].pos.w));
            o[4] = float(val(b[size_t(i)].vel.x)); o[5] = float(val(b[size_t(i)].vel.y)); o[6] = float(val(b[size_t(i)].vel.z)); o[7] = float(val(b[size_t(i)].vel.w));
        }
    }
    return 0;
}

thread_local std::string g_err;

}  // namespace
}  // namespace grad

extern "C" {

const char* grad_last_error() { return grad::g_err.c_str(); }

// One run of `steps` steps from `state` (n GpuBoids) on a grid venue; returns the loss, its derivatives along nt
// directions (dr, dv0: nt x n, dtau: nt; nt <= 8) and the branch signature; stateOut (n x 8, may be null) the end
// state. prec 32: float arithmetic (nt 0: the plain float step; nt > 0: float primal, double tangents);
// prec 64: double arithmetic.
int grad_eval(int prec, const SwarmParams* p, const SwarmVenue* v, const float* state, int n, const double* radius, const double* v0,
              double tau, int steps, int threads, int nt, const double* dr, const double* dv0, const double* dtau, double* loss,
              double* dloss, uint64_t* sig, float* stateOut) {
    using namespace grad;
    if (!p || !v || !state || !radius || !v0 || !loss || n <= 0 || steps < 0 || nt < 0 || nt > 8) { g_err = "invalid argument"; return -1; }
    if (v->kind != SWARM_VENUE_GRID || !v->wall_sdf || !v->nav_dist) { g_err = "grid venues only"; return -1; }
    const int th = threads > 0 ? threads : omp_get_max_threads();
    if (prec == 32) {
        if (nt == 0) return runT<float>(*p, *v, state, n, radius, v0, tau, steps, th, 0, nullptr, nullptr, nullptr, loss, nullptr, sig, stateOut);
        if (nt == 1) return runT<Dual<float, 1>>(*p, *v, state, n, radius, v0, tau, steps, th, nt, dr, dv0, dtau, loss, dloss, sig, stateOut);
        if (nt <= 4) return runT<Dual<float, 4>>(*p, *v, state, n, radius, v0, tau, steps, th, nt, dr, dv0, dtau, loss, dloss, sig, stateOut);
        return runT<Dual<float, 8>>(*p, *v, state, n, radius, v0, tau, steps, th, nt, dr, dv0, dtau, loss, dloss, sig, stateOut);
    }
    if (prec == 64) {
        if (nt == 0) return runT<double>(*p, *v, state, n, radius, v0, tau, steps, th, 0, nullptr, nullptr, nullptr, loss, nullptr, sig, stateOut);
        if (nt == 1) return runT<Dual<double, 1>>(*p, *v, state, n, radius, v0, tau, steps, th, nt, dr, dv0, dtau, loss, dloss, sig, stateOut);
        if (nt <= 4) return runT<Dual<double, 4>>(*p, *v, state, n, radius, v0, tau, steps, th, nt, dr, dv0, dtau, loss, dloss, sig, stateOut);
        return runT<Dual<double, 8>>(*p, *v, state, n, radius, v0, tau, steps, th, nt, dr, dv0, dtau, loss, dloss, sig, stateOut);
    }
    g_err = "prec must be 32 or 64";
    return -1;
}

}  // extern "C"
