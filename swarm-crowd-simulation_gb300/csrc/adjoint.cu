// The adjoint of the crowd step on a grid venue: reverse-mode derivatives written by hand, kernel by kernel, against
// the forward of step_kernels.cu (DedovSergei/swarm-crowd-simulation src/cpu_crowd_sim.cpp: predict :655-777,
// projectSlot :781-822, finalPass :835-866; the analytic-venue static contacts :291-297, :386-399, :444-447, :465-514).
//
// Loss: L = dt * sum_t sum_{i active after step t} D(p_i(t)), D the bilinear sample of the geodesic distance grid.
// Parameters: each agent's radius r_i and desired speed v0_i, the relaxation time tau (relax_step = exp(-dt / tau)).
//
// The branches are frozen at the forward's choices: every comparison (contact activation, the headway cone and
// argmin, the clamps, the speed cap, the wall passes, the plane test, exits) is re-evaluated on the taped forward
// values with the forward's own arithmetic, so it takes the same side, and only the arithmetic between branches is
// differentiated. Pairs are reversed by gathering, not scattering: the contact relation and the separation pairs are
// symmetric and their Jacobians even in the offset, so slot s collects sum_m G(o_sm) (lambda_s - lambda_m) from its
// own neighbour loop. Every adjoint value is written by one thread, so the gradients are deterministic.
//
//   k_adj_final    per slot: the final pass's static contacts reversed (recomputed from the tape), the loss term of
//                  the step's result, the own terms of the last sweep; agents inactive at the step pass their adjoint on
//   k_adj_sweep    sweep k (k = K .. 1): the neighbour gather of the contact-sum adjoints, then the own terms of sweep
//                  k - 1 (cap, wall plane)
//   k_adj_predict  predict's own terms: static contacts, speed cap, along-goal clip, relaxation, obstacle push,
//                  direction, headway clamp, e_goal (the separation sum and sAhead come from the tape)
//   k_adj_gather   predict's pair terms (separation, the headway argmin) gathered over the perception disk; writes the
//                  state adjoint before the step and the radius gradient
//   k_adj_step_fused  the four as one persistent cooperative launch (K + 2 grid barriers), the neighbour gathers
//                  split over ADJ_LANES lanes per slot
#include "adjoint.cuh"

#include <algorithm>

#include <cuda/atomic>

#include "device_math.cuh"
#include "venue_grid.cuh"

namespace swarm_gpu {
namespace {

// ---- the wall query with its derivative data: the same arithmetic as GridVenue::wall ----
struct WallD {
    f2 n;        // unit normal (0 when |g| <= eps)
    float d;     // distance; WALL_NONE: none within reach or outside the field (a constant: no derivative)
    f2 g;        // d d / d p, the bilinear gradient
    float gl;    // |g|
    float m;     // d g.x / d p.y = d g.y / d p.x
};

__device__ WallD wallD(const SwarmParams& P, const VenueArgs& V, f2 p, float reach) {
    WallD w;
    w.n = f2{0.0f, 0.0f};
    w.d = WALL_NONE;
    w.g = f2{0.0f, 0.0f};
    w.gl = 0.0f;
    w.m = 0.0f;
    const float fx = (p.x - V.wox) * V.winv, fy = (p.y - V.woy) * V.winv;
    if (!(fx >= 0.0f && fy >= 0.0f && fx <= float(V.wnx - 1) && fy <= float(V.wny - 1))) return w;
    const int ix = smin(int(floorf(fx)), V.wnx - 2), iy = smin(int(floorf(fy)), V.wny - 2);
    const float wx = fx - float(ix), wy = fy - float(iy);
    const size_t r0 = size_t(iy) * size_t(V.wnx) + size_t(ix), r1 = r0 + size_t(V.wnx);
    const float c00 = __ldg(V.wall + r0), c10 = __ldg(V.wall + r0 + 1), c01 = __ldg(V.wall + r1), c11 = __ldg(V.wall + r1 + 1);
    const float d = mix(mix(c00, c10, wx), mix(c01, c11, wx), wy);
    if (d >= reach) return w;
    const f2 g{mix(c10 - c00, c11 - c01, wy) * V.winv, mix(c01 - c00, c11 - c10, wx) * V.winv};
    w.gl = length(g);
    w.n = w.gl > P.safe_eps ? g / w.gl : f2{0.0f, 0.0f};
    w.d = d;
    w.g = g;
    w.m = ((c11 - c01) - (c10 - c00)) * V.winv * V.winv;
    return w;
}

// The adjoint of p from the adjoints of a wall query's (normal, distance)
__device__ __forceinline__ f2 wallBack(const WallD& w, f2 lamN, float lamD) {
    f2 r{w.g.x * lamD, w.g.y * lamD};
    if (nonzero(w.n)) {
        const float nl = dot(w.n, lamN);
        const f2 mu{(lamN.x - w.n.x * nl) / w.gl, (lamN.y - w.n.y * nl) / w.gl};
        r.x += w.m * mu.y;
        r.y += w.m * mu.x;
    }
    return r;
}

// ---- the distance grid: value, e_goal (as GridVenue::goal) and derivative data ----
struct NavD {
    float D;     // the bilinear value (the loss sample)
    f2 e;        // e_goal
    f2 g;        // the bilinear gradient in cell units (e = -g / |g|)
    float gl;
    float m;     // d g.x / d wy = d g.y / d wx
    float sx, sy;   // d wx / d p.x, d wy / d p.y (0 where the coordinate was clamped)
};

__device__ NavD navD(const SwarmParams& P, const VenueArgs& V, f2 p) {
    NavD q;
    float fx = (p.x - V.nox) * V.ninv, fy = (p.y - V.noy) * V.ninv;
    q.sx = (fx < 0.0f || float(V.nnx - 1) < fx) ? 0.0f : V.ninv;
    q.sy = (fy < 0.0f || float(V.nny - 1) < fy) ? 0.0f : V.ninv;
    fx = sclamp(fx, 0.0f, float(V.nnx - 1));
    fy = sclamp(fy, 0.0f, float(V.nny - 1));
    const int ix = smin(int(floorf(fx)), V.nnx - 2), iy = smin(int(floorf(fy)), V.nny - 2);
    const float wx = fx - float(ix), wy = fy - float(iy);
    const size_t r0 = size_t(iy) * size_t(V.nnx) + size_t(ix), r1 = r0 + size_t(V.nnx);
    const float d00 = __ldg(V.nav + r0), d10 = __ldg(V.nav + r0 + 1), d01 = __ldg(V.nav + r1), d11 = __ldg(V.nav + r1 + 1);
    q.D = mix(mix(d00, d10, wx), mix(d01, d11, wx), wy);
    q.g = f2{mix(d10 - d00, d11 - d01, wy), mix(d01 - d00, d11 - d10, wx)};
    q.e = safeNormalize(f2{-q.g.x, -q.g.y}, P.safe_eps);
    q.gl = length(q.g);
    q.m = (d11 - d01) - (d10 - d00);
    return q;
}

// ---- the static contacts, recorded for the reverse pass ----
enum : uint8_t { OP_FLOOR = 1, OP_SWEEP = 2, OP_WALL = 3 };
// A wall pass: a = the position it queried, b = the velocity before it; flags 1 pushed, 2 velocity clipped.
// A floor contact: flags 1 fired. A sweep back: a, b as above, lo the bisection's result, flags 1 velocity clipped.
struct SOp {
    uint8_t kind, flags;
    f2 a, b;
    float lo;
};
constexpr int MAX_SOPS = 16;   // 4 floor contacts + a sweep back + 2 x wall_passes (<= 5)
struct STape {
    SOp op[MAX_SOPS];
    int nops;
    int wallOp;       // the wall pass whose query gave the recorded wall (-1: none)
    bool wallBreak;   // recorded as (n, d - r) by a pass that stopped, else (n, 0) by a pass that pushed
};

__device__ __forceinline__ void pushOp(STape& T, uint8_t kind, uint8_t flags, f2 a, f2 b, float lo) {
    if (T.nops < MAX_SOPS) T.op[T.nops] = SOp{kind, flags, a, b, lo};
    ++T.nops;
}

__device__ bool recRest(const GridVenue& ven, STape& T, f3& np, f3& nv, float zFrom, float r) {
    const bool f = ven.restOnFloor(np, nv, zFrom, r);
    pushOp(T, OP_FLOOR, f ? 1 : 0, f2{0.0f, 0.0f}, f2{0.0f, 0.0f}, 0.0f);
    return f;
}
__device__ bool recSettle(const GridVenue& ven, STape& T, f3& np, f3& nv, float zFrom, float r) {
    const bool f = ven.settleOnFloor(np, nv, zFrom, r);
    pushOp(T, OP_FLOOR, f ? 1 : 0, f2{0.0f, 0.0f}, f2{0.0f, 0.0f}, 0.0f);
    return f;
}
// GridVenue::sweepBack, recorded
__device__ bool recSweep(const GridVenue& ven, STape& T, f3 pOld, f3& np, f3& nv) {
    const SwarmParams& P = ven.P;
    if (!ven.solid(np)) return false;
    float lo = 0.0f, hi = 1.0f;
    if (!ven.solid(f3{np.x, np.y, pOld.z})) lo = 1.0f;
    for (int i = 0; i < P.sweep_bisections; ++i) {
        float t = 0.5f * (lo + hi);
        f2 m = mix(xy(pOld), xy(np), t);
        if (ven.solid(f3{m.x, m.y, pOld.z})) hi = t;
        else lo = t;
    }
    const f2 a = xy(np), b = xy(nv);
    f2 d = safeNormalize(xy(np) - xy(pOld), P.safe_eps);
    f2 m = mix(xy(pOld), xy(np), lo);
    np = f3{m.x, m.y, pOld.z};
    float vd = dot(xy(nv), d);
    if (vd > 0.0f) setXY(nv, xy(nv) - d * vd);
    nv.z = 0.0f;
    pushOp(T, OP_SWEEP, vd > 0.0f ? 1 : 0, a, b, lo);
    return true;
}
// GridVenue::clearWalls, recorded; op / brk: the pass that recorded the returned wall
__device__ bool recClear(const GridVenue& ven, STape& T, f3& np, f3& nv, f3& wallOut, float r, int& op, bool& brk) {
    const SwarmParams& P = ven.P;
    bool moved = false;
    wallOut = f3{0.0f, 0.0f, 0.0f};
    op = -1;
    brk = false;
    for (int pass = 0; pass < P.wall_passes; ++pass) {
        const int idx = T.nops;
        const f2 a = xy(np), b = xy(nv);
        const f3 w = ven.wall(xy(np), P.feeler_reach);
        if (w.z >= r) {
            if (w.z < WALL_NONE) { wallOut = f3{w.x, w.y, w.z - r}; op = idx; brk = true; }
            pushOp(T, OP_WALL, 0, a, b, 0.0f);
            break;
        }
        setXY(np, xy(np) + f2{w.x, w.y} * (r - w.z));
        moved = true;
        wallOut = f3{w.x, w.y, 0.0f};
        op = idx;
        brk = false;
        const float vDotN = dot(xy(nv), f2{w.x, w.y});
        if (vDotN < 0.0f) setXY(nv, xy(nv) - f2{w.x, w.y} * vDotN);
        pushOp(T, OP_WALL, vDotN < 0.0f ? 3 : 1, a, b, 0.0f);
    }
    return moved;
}
// GridVenue::resolveStatic, recorded
__device__ bool recResolve(const GridVenue& ven, STape& T, f3 pOld, f3& np, f3& nv, bool settle, f3& wallOut, float r) {
    T.nops = 0;
    bool grounded = settle ? recSettle(ven, T, np, nv, pOld.z, r) : recRest(ven, T, np, nv, pOld.z, r);
    if (!grounded && recSweep(ven, T, pOld, np, nv)) grounded = recRest(ven, T, np, nv, pOld.z, r);
    int op1;
    bool br1;
    const bool walls = recClear(ven, T, np, nv, wallOut, r, op1, br1);
    T.wallOp = op1;
    T.wallBreak = br1;
    if (walls) {
        if (grounded) {
            recSettle(ven, T, np, nv, pOld.z, r);
            f3 w2;
            int op2;
            bool br2;
            const bool again = recClear(ven, T, np, nv, w2, r, op2, br2);
            if (w2.x != 0.0f || w2.y != 0.0f) { wallOut = w2; T.wallOp = op2; T.wallBreak = br2; }
            if (again) recRest(ven, T, np, nv, pOld.z, r);
        } else {
            recRest(ven, T, np, nv, pOld.z, r);
        }
    }
    return grounded;
}

// The static contacts reversed: (lnp, lnv) the adjoints of the result in, of the input out; lWallN / lWallZ the
// adjoint of the recorded wall (normal, offset); lr and lpOld accumulate
__device__ void revStatics(const SwarmParams& P, const VenueArgs& V, const STape& T, f3 pOld, float r, f2 lWallN, float lWallZ,
                           f3& lnp, f3& lnv, float& lr, f3& lpOld) {
    const int nops = T.nops < MAX_SOPS ? T.nops : MAX_SOPS;
    for (int i = nops - 1; i >= 0; --i) {
        const SOp o = T.op[i];
        if (o.kind == OP_FLOOR) {
            if (o.flags) {   // np.z = floor + r, nv.z = 0
                lr += lnp.z;
                lnp.z = 0.0f;
                lnv.z = 0.0f;
            }
        } else if (o.kind == OP_WALL) {
            f2 lamN{0.0f, 0.0f};
            float lamD = 0.0f;
            if (i == T.wallOp) {
                lamN = lWallN;
                if (T.wallBreak) { lamD = lWallZ; lr -= lWallZ; }
            }
            if (o.flags & 1) {   // np += n (r - d); nv -= n (nv . n) when clipped
                const WallD w = wallD(P, V, o.a, P.feeler_reach);
                const f2 ln = xy(lnp);
                lamN = lamN + ln * (r - w.d);
                const float nl = dot(w.n, ln);
                lr += nl;
                lamD -= nl;
                if (o.flags & 2) {
                    const f2 lv = xy(lnv);
                    const float vdn = dot(o.b, w.n), lvn = dot(w.n, lv);
                    lamN = lamN - lv * vdn - o.b * lvn;
                    setXY(lnv, lv - w.n * lvn);
                }
                setXY(lnp, xy(lnp) + wallBack(w, lamN, lamD));
            } else if (i == T.wallOp) {
                const WallD w = wallD(P, V, o.a, P.feeler_reach);
                if (w.d < WALL_NONE) setXY(lnp, xy(lnp) + wallBack(w, lamN, lamD));
            }
        } else {   // sweep back: np = (mix(pOld, a, lo), pOld.z); nv -= d (nv . d) when clipped; nv.z = 0
            const f2 e = o.a - xy(pOld);
            const float el = length(e);
            const f2 d = el > P.safe_eps ? e / el : f2{0.0f, 0.0f};
            f2 la{0.0f, 0.0f};
            if (o.flags & 1) {
                const f2 lv = xy(lnv);
                const float vd = dot(o.b, d), ldv = dot(d, lv);
                const f2 ld = -(lv * vd) - o.b * ldv;
                setXY(lnv, lv - d * ldv);
                if (el > P.safe_eps) {
                    const f2 le = (ld - d * dot(d, ld)) / el;
                    la = la + le;
                    lpOld.x -= le.x;
                    lpOld.y -= le.y;
                }
            }
            lnv.z = 0.0f;
            la = la + xy(lnp) * o.lo;
            lpOld.x += lnp.x * (1.0f - o.lo);
            lpOld.y += lnp.y * (1.0f - o.lo);
            lpOld.z += lnp.z;
            lnp = f3{la.x, la.y, 0.0f};
        }
    }
}

__device__ __forceinline__ int activeCount(const AdjArgs& A) { return int(A.start[A.V.ncells]); }

// The own part of sweep k of slot s reversed: lq the adjoint of its result (xy); returns the adjoint of its input
// through the identity path, stores the adjoint of its contact sum, adds the wall plane's adjoint
__device__ f2 sweepOwnBack(const AdjArgs& A, int s, int k, f2 lq, float2* lamCOut, float4 plane, float4& lplane) {
    const SwarmParams& P = A.P;
    const float4 qin = A.f4[A.L.q(k - 1) + size_t(s)];
    const float4 c = A.f4[A.L.corr(k) + size_t(s)];
    const f2 corr{c.x, c.y};
    const float len = length(corr);
    const bool capped = len > P.proj_max_shift;
    const f2 cc = capped ? corr * (P.proj_max_shift / len) : corr;
    const f2 q1 = xy(qin) + cc;
    f2 l1 = lq;
    if (plane.w == PLANE_WALL || plane.w == PLANE_WALL + PLANE_GROUNDED) {
        const f2 n{plane.x, plane.y};
        const float sd = plane.z - dot(q1, n);
        if (sd > 0.0f) {   // q'' = q' + n (offset - n . q')
            const float nl = dot(n, lq);
            l1 = lq - n * nl;
            lplane.x += sd * lq.x - nl * q1.x;
            lplane.y += sd * lq.y - nl * q1.y;
            lplane.z += nl;
        }
    }
    f2 lcs = l1;
    if (capped) {
        const f2 u = corr / len;
        lcs = (l1 - u * dot(u, l1)) * (P.proj_max_shift / len);
    }
    const float a = P.proj_relax / float(smax(int(c.z), 1));
    lamCOut[s] = make_float2(lcs.x * a, lcs.y * a);
    return l1;
}

// The final pass of slot s reversed; returns D of its result (0 unless it stays active)
__device__ double adjFinalSlot(const AdjArgs& A, int s) {
    const SwarmParams& P = A.P;
    const VenueArgs& V = A.V;
    const TapeLayout& L = A.L;
    const uint32_t id = A.sid[s];
    if (s >= activeCount(A)) {   // inactive at the step: carried over unchanged
        A.lamOut[2 * size_t(id)] = A.lamIn[2 * size_t(id)];
        A.lamOut[2 * size_t(id) + 1] = A.lamIn[2 * size_t(id) + 1];
        return 0.0;
    }
    const float4 q0 = A.f4[L.q(0) + size_t(s)];
    const float4 zero = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (q0.w < 0.0f) {   // parked this step: its result is a constant
        A.lamQ[s] = zero;
        A.lamNv[s] = zero;
        A.lamPOld[s] = zero;
        A.lamPlane[s] = zero;
        A.lamR[s] = 0.0f;
        return 0.0;
    }
    const GridVenue ven{P, V};
    const int K = L.K;
    const float4 b = K > 0 ? A.f4[L.qK() + size_t(s)] : q0;
    f3 np = xyz(b), nv = xyz(A.f4[L.vel1() + size_t(s)]);
    const f3 pOld = xyz(A.f4[L.pos0() + size_t(s)]);
    const float ri = A.prm[s].x;
    const float4 plane = A.f4[L.plane() + size_t(s)];
    STape T;
    T.nops = 0;
    const bool moved = b.w > 0.0f;
    if (moved) {
        f3 wl;
        recResolve(ven, T, pOld, np, nv, plane.w >= PLANE_GROUNDED, wl, ri);
    }
    // the loss term of the result, and its adjoint
    const NavD nd = navD(P, V, xy(np));
    const float4 lp = A.lamIn[2 * size_t(id)], lv = A.lamIn[2 * size_t(id) + 1];
    f3 lnp{lp.x + P.dt * nd.g.x * nd.sx, lp.y + P.dt * nd.g.y * nd.sy, lp.z};
    f3 lnv{lv.x, lv.y, lv.z};
    float lr = 0.0f;
    f3 lpOld{0.0f, 0.0f, 0.0f};
    if (moved) revStatics(P, V, T, pOld, ri, f2{0.0f, 0.0f}, 0.0f, lnp, lnv, lr, lpOld);
    float4 lplane = zero;
    f2 lq = xy(lnp);
    if (K > 0) lq = sweepOwnBack(A, s, K, lq, A.lamC[K & 1], plane, lplane);
    A.lamQ[s] = make_float4(lq.x, lq.y, lnp.z, 0.0f);
    A.lamNv[s] = make_float4(lnv.x, lnv.y, lnv.z, 0.0f);
    A.lamPOld[s] = make_float4(lpOld.x, lpOld.y, lpOld.z, 0.0f);
    A.lamPlane[s] = lplane;
    A.lamR[s] = lr;
    return double(nd.D);
}

// A block's sum of v in a fixed order (warp trees, then the warps in order); valid in thread 0
template <int THREADS>
__device__ __forceinline__ double blockSum(double v, double* warpSum) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31u) == 0) warpSum[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)   // the block's warps (THREADS: the most a block of this kernel has)
        for (int w = 0; w < int(blockDim.x >> 5) && w < THREADS / 32; ++w) t += warpSum[w];
    __syncthreads();
    return t;
}

__global__ void __launch_bounds__(ADJ_FINAL_THREADS) k_adj_final(AdjArgs A) {
    __shared__ double warpSum[ADJ_FINAL_THREADS / 32];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const double d = s < A.L.n ? adjFinalSlot(A, s) : 0.0;
    const double t = blockSum<ADJ_FINAL_THREADS>(d, warpSum);
    if (threadIdx.x == 0) A.lossPart[blockIdx.x] = t;
}

// Sums v over the G consecutive lanes of a lane group (every lane of the warp calls it; all get the same bits)
template <int G>
__device__ __forceinline__ float groupSum(float v) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// The 3 x 3 neighbour rows of a slot: slot ranges [rk0[j], rk1[j])
__device__ __forceinline__ void rows3(const AdjArgs& A, uint32_t cid, uint32_t* rk0, uint32_t* rk1) {
    const VenueArgs& V = A.V;
    const int resX = V.resX, resY = V.resY;
    const int cx = int(cid % uint32_t(resX)), cy = int(cid / uint32_t(resX));
    const int xlo = max(cx - 1, 0), xhi = min(cx + 1, resX - 1);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const int ny = cy + j - 1;
        const bool ok = ny >= 0 && ny < resY;
        rk0[j] = ok ? A.start[xlo + ny * resX] : 0u;
        rk1[j] = ok ? A.start[xhi + 1 + ny * resX] : 0u;
    }
}

// Sweep k of slot s reversed by a group of G lanes (lane = 0 .. G - 1; every lane of the warp takes part): the
// neighbour gather split over the lanes, summed, then lane 0 adds the identity path and reverses the own part of
// sweep k - 1. valid: s is active and not parked.
// rows: the slot's 3 x 3 neighbour rows when the caller holds them (null: looked up)
template <int G>
__device__ void adjSweepSlot(const AdjArgs& A, int s, int lane, bool valid, int k, const uint32_t* rows = nullptr) {
    const SwarmParams& P = A.P;
    const TapeLayout& L = A.L;
    const float4* q = A.f4 + L.q(k - 1);
    const float2* lc = A.lamC[k & 1];
    float4 b = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    float2 lcs = make_float2(0.0f, 0.0f);
    float ri = 0.0f;
    uint32_t rk0[3] = {0u, 0u, 0u}, rk1[3] = {0u, 0u, 0u};
    if (valid) {
        b = q[s];
        lcs = lc[s];
        ri = A.prm[s].x;
        if (rows) {
#pragma unroll
            for (int j = 0; j < 3; ++j) { rk0[j] = rows[j]; rk1[j] = rows[3 + j]; }
        } else {
            rows3(A, A.skey[s], rk0, rk1);
        }
    }
    const uint32_t len0 = rk1[0] - rk0[0], len1 = rk1[1] - rk0[1], total = len0 + len1 + (rk1[2] - rk0[2]);
    f2 lq{0.0f, 0.0f};
    float lr = 0.0f;
    for (uint32_t idx = uint32_t(lane); idx < total; idx += uint32_t(G)) {
        const uint32_t m = idx < len0 ? rk0[0] + idx : (idx < len0 + len1 ? rk0[1] + (idx - len0) : rk0[2] + (idx - len0 - len1));
        if (int(m) == s) continue;
        const float4 op = q[m];
        const float rj = A.prm[m].x;
        const f3 offset = xyz(b) - xyz(op);
        const float dc = ri + rj, dc2 = dc * dc;
        const float dxy2 = dot(xy(offset), xy(offset));
        if (op.w >= 0.0f && fabsf(offset.z) < dc && dxy2 < dc2) {
            const float2 lcm = lc[m];
            const f2 dl{lcs.x - lcm.x, lcs.y - lcm.y};
            if (dxy2 <= P.stacked_xy2) {
                const f2 dir = pairDirection(A.sid[s], A.sid[m], P.hash_to_radians);
                lr += 0.5f * dot(dir, dl);
            } else {
                // g = (dc / d - 1) o / 2: dg/do = ((dc / d - 1) I - (dc / d) oh oh^T) / 2, dg/ddc = oh / 2
                const float d = sqrtf(dxy2);
                const f2 oh = xy(offset) / d;
                const float ohl = dot(oh, dl);
                const float t = dc / d;
                lq.x += 0.5f * ((t - 1.0f) * dl.x - t * oh.x * ohl);
                lq.y += 0.5f * ((t - 1.0f) * dl.y - t * oh.y * ohl);
                lr += 0.5f * ohl;
            }
        }
    }
    lq.x = groupSum<G>(lq.x);
    lq.y = groupSum<G>(lq.y);
    lr = groupSum<G>(lr);
    if (!valid || lane != 0) return;
    const float4 lq4 = A.lamQ[s];
    lq.x += lq4.x;
    lq.y += lq4.y;
    if (k > 1) {
        float4 lplane = A.lamPlane[s];
        lq = sweepOwnBack(A, s, k - 1, lq, A.lamC[(k - 1) & 1], A.f4[L.plane() + size_t(s)], lplane);
        A.lamPlane[s] = lplane;
    }
    A.lamQ[s] = make_float4(lq.x, lq.y, lq4.z, 0.0f);
    A.lamR[s] += lr;
}

__device__ __forceinline__ bool sweepsSlot(const AdjArgs& A, int s) {   // active and not parked this step
    return s < A.L.n && s < activeCount(A) && A.f4[A.L.q(0) + size_t(s)].w >= 0.0f;
}

__global__ void __launch_bounds__(128) k_adj_sweep(AdjArgs A) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    adjSweepSlot<1>(A, s, 0, sweepsSlot(A, s), A.sweep);
}

// Predict's own terms of slot s reversed (the separation sum and sAhead from the tape)
__device__ void adjPredictSlot(const AdjArgs& A, int s) {
    const SwarmParams& P = A.P;
    const VenueArgs& V = A.V;
    const TapeLayout& L = A.L;
    const float4 zero = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (A.f4[L.q(0) + size_t(s)].w < 0.0f) {   // parked this step: predict produced a constant
        A.lamSep[s] = zero;
        A.lamP[s] = zero;
        A.lamV[s] = zero;
        return;
    }
    const GridVenue ven{P, V};
    const uint32_t id = A.sid[s];
    const float4 p = A.f4[L.pos0() + size_t(s)], v = A.f4[L.vel0() + size_t(s)];
    const float2 pr = A.prm[s];
    const float ri = pr.x;
    const float4 rec = A.f4[L.pred() + size_t(s)];
    const f2 sep{rec.x, rec.y};
    const float sAhead = rec.z;
    const int jstar = __float_as_int(rec.w);

    // ---- predict's forward after the neighbour loop (the expressions of predictItem) ----
    const NavD nq = navD(P, V, xy(p));
    const f2 eGoal = nq.e;
    const float sf = ven.speedFactor(xyz(p));
    const float vFree = pr.y * sf;
    const float hw = sAhead * P.headway_rate;
    const int clampBranch = hw < 0.0f ? 0 : (vFree < hw ? 2 : 1);
    const float vDes0 = sclamp(hw, 0.0f, vFree);
    const float le = length(eGoal);
    const float vDes = vDes0 * le;
    const f2 u = eGoal + sep;
    const float ul = length(u);
    const f2 eDir = safeNormalize(u, P.safe_eps);

    const f3 torso{p.x + 0.0f, p.y + 0.0f, p.z + P.torso_height};
    const WallD wT = wallD(P, V, xy(torso), WALL_NONE);
    const float fT = torso.z - ven.floorHeight(xy(torso));
    const bool tFloor = fT < wT.d;
    const float dTorso = tFloor ? fT : wT.d;
    const f3 ks[4] = {f3{1.0f, -1.0f, -1.0f}, f3{-1.0f, -1.0f, 1.0f}, f3{-1.0f, 1.0f, -1.0f}, f3{1.0f, 1.0f, 1.0f}};
    f2 aObs{0.0f, 0.0f}, ah{0.0f, 0.0f};
    f3 nrm3{0.0f, 0.0f, 0.0f};
    float G3l = 0.0f, nl = 0.0f;
    bool obsOn = false;
    if (dTorso < P.obstacle_range) {
        const float h = P.obstacle_grad_h;
        float mk[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) mk[k] = ven.map(torso + ks[k] * h);
        const f3 G3 = (ks[0] * mk[0] + ks[1] * mk[1] + ks[2] * mk[2] + ks[3] * mk[3]) * P.obstacle_grad_scale;
        G3l = length(G3);
        nrm3 = safeNormalize(G3, P.safe_eps);
        const f2 nrm = xy(nrm3);
        nl = length(nrm);
        if (nl > P.obstacle_min_normal) {
            ah = safeNormalize(nrm, P.safe_eps);
            aObs = ah * (P.obstacle_range - dTorso) * P.w_obs * P.obstacle_gain;
            obsOn = true;
        }
    }
    const f2 vEq = eDir * vDes + aObs * P.tau_relax;
    f3 nv = xyz(v);
    const f2 v2 = xy(nv);
    setXY(nv, vEq + (xy(nv) - vEq) * P.relax_step);
    const f2 nvA = xy(nv);
    const float along = dot(xy(nv), eGoal);
    const bool alongOn = along > vDes;
    if (alongOn) setXY(nv, xy(nv) - eGoal * (along - vDes));
    const f2 nvB = xy(nv);
    nv.z -= P.gravity_dt;
    const bool vzKept = !(0.0f < nv.z);
    nv.z = smin(nv.z, 0.0f);
    const float spd = length(xy(nv));
    const bool capOn = spd > P.v_max;
    if (capOn) setXY(nv, safeNormalize(xy(nv), P.safe_eps) * P.v_max);
    f3 np = xyz(p) + nv * P.dt;
    STape T;
    f3 wl;
    recResolve(ven, T, xyz(p), np, nv, false, wl, ri);
    bool probe = false;
    WallD wp;
    if (wl.x == 0.0f && wl.y == 0.0f) {
        probe = true;
        T.wallOp = -1;
        wp = wallD(P, V, xy(np), P.plane_probe_reach);
        wl = wp.d >= 0.0f && wp.d < WALL_NONE ? f3{wp.n.x, wp.n.y, smax(wp.d - ri, 0.0f)} : f3{0.0f, 0.0f, 0.0f};
    }

    // ---- reverse ----
    const float4 lq = A.lamQ[s], lnv4 = A.lamNv[s], lpl = A.lamPlane[s], lpo = A.lamPOld[s];
    f3 lnp{lq.x, lq.y, lq.z}, lnv{lnv4.x, lnv4.y, lnv4.z};
    f3 lp{lpo.x, lpo.y, lpo.z}, lv{0.0f, 0.0f, 0.0f};
    float lr = 0.0f;
    // plane = (wn, np . wn - wall offset)
    f2 lwn{lpl.x + lpl.z * np.x, lpl.y + lpl.z * np.y};
    lnp.x += lpl.z * wl.x;
    lnp.y += lpl.z * wl.y;
    float lwz = -lpl.z;
    if (probe) {
        if (wp.d >= 0.0f && wp.d < WALL_NONE) {
            float lD = 0.0f;
            if (!(wp.d - ri < 0.0f)) { lD = lwz; lr -= lwz; }
            setXY(lnp, xy(lnp) + wallBack(wp, lwn, lD));
        }
        lwn = f2{0.0f, 0.0f};
        lwz = 0.0f;
    }
    f3 lpOld{0.0f, 0.0f, 0.0f};
    revStatics(P, V, T, xyz(p), ri, lwn, lwz, lnp, lnv, lr, lpOld);
    lp = lp + lpOld;
    // np = p + nv dt
    lp = lp + lnp;
    lnv = lnv + lnp * P.dt;
    // the speed cap: nv = v_max nv / |nv|
    f2 lnx = xy(lnv);
    if (capOn) {
        const f2 nh = nvB / spd;
        lnx = (lnx - nh * dot(nh, lnx)) * (P.v_max / spd);
    }
    if (vzKept) lv.z += lnv.z;
    // the clip along e_goal: nv = nvA - e (e . nvA - vDes)
    f2 leG{0.0f, 0.0f};
    float lvDes = 0.0f;
    if (alongOn) {
        const float el2 = dot(eGoal, lnx);
        leG = leG - lnx * (along - vDes) - nvA * el2;
        lvDes += el2;
        lnx = lnx - eGoal * el2;
    }
    // relaxation: nv = vEq + (v - vEq) rho
    const float rho = P.relax_step;
    const f2 lvEq = lnx * (1.0f - rho);
    lv.x += lnx.x * rho;
    lv.y += lnx.y * rho;
    const float lrho = dot(v2 - vEq, lnx);
    // vEq = eDir vDes + aObs tau
    const f2 leDir = lvEq * vDes;
    lvDes += dot(eDir, lvEq);
    const f2 laObs = lvEq * P.tau_relax;
    const double ltau = double(dot(aObs, lvEq)) + double(lrho) * double(rho) * double(P.dt) / (double(P.tau_relax) * double(P.tau_relax));
    // the obstacle push: aObs = ah (range - dTorso) w_obs gain, ah = normalize(xy(normalize(G3)))
    if (obsOn) {
        const float S = (P.obstacle_range - dTorso) * P.w_obs * P.obstacle_gain;
        const f2 lah = laObs * S;
        const float ldT = -dot(ah, laObs) * P.w_obs * P.obstacle_gain;
        const f2 lnrm = (lah - ah * dot(ah, lah)) / nl;
        const f3 ln3{lnrm.x, lnrm.y, 0.0f};
        const float nd3 = dot(nrm3, ln3);
        const f3 lG3{(ln3.x - nrm3.x * nd3) / G3l, (ln3.y - nrm3.y * nd3) / G3l, (ln3.z - nrm3.z * nd3) / G3l};
        const float h = P.obstacle_grad_h;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float lm = P.obstacle_grad_scale * dot(ks[k], lG3);
            const f3 pk = torso + ks[k] * h;
            const WallD wk = wallD(P, V, xy(pk), WALL_NONE);
            const float fk = pk.z - ven.floorHeight(xy(pk));
            if (fk < wk.d) lp.z += lm;
            else if (wk.d < WALL_NONE) { lp.x += wk.g.x * lm; lp.y += wk.g.y * lm; }
        }
        if (tFloor) lp.z += ldT;
        else if (wT.d < WALL_NONE) { lp.x += wT.g.x * ldT; lp.y += wT.g.y * ldT; }
    }
    // eDir = normalize(eGoal + sep)
    f2 lu{0.0f, 0.0f};
    if (ul > P.safe_eps) lu = (leDir - eDir * dot(eDir, leDir)) / ul;
    leG = leG + lu;
    // vDes = clamp(sAhead rate, 0, vFree) |eGoal|
    const float lvDes0 = lvDes * le;
    if (le > 0.0f) leG = leG + eGoal * (vDes0 * lvDes / le);
    float lsA = 0.0f, lv0 = 0.0f;
    if (clampBranch == 1) lsA = lvDes0 * P.headway_rate;
    else if (clampBranch == 2) lv0 = lvDes0 * sf;
    // e_goal = -g / |g|
    if (nq.gl > P.safe_eps) {
        const f2 lg = -((leG - eGoal * dot(eGoal, leG)) / nq.gl);
        lp.x += nq.m * nq.sx * lg.y;
        lp.y += nq.m * nq.sy * lg.x;
    }
    // sAhead = |p - p_j*| - r - r_j*: the own terms (the argmin's, in its gather)
    if (jstar >= 0 && lsA != 0.0f) {
        const float4 pj = A.f4[L.pos0() + size_t(jstar)];
        const f2 o{p.x - pj.x, p.y - pj.y};
        const float dxy = sqrtf(dot(o, o));
        if (dxy > 0.0f) { lp.x += o.x / dxy * lsA; lp.y += o.y / dxy * lsA; }
        lr -= lsA;
    }
    A.lamSep[s] = make_float4(lu.x, lu.y, lsA, 0.0f);
    A.lamP[s] = make_float4(lp.x, lp.y, lp.z, 0.0f);
    A.lamV[s] = make_float4(lv.x, lv.y, lv.z, 0.0f);
    A.lamR[s] += lr;
    A.gV0[id] += double(lv0);
    A.gTau[id] += ltau;
}

__global__ void __launch_bounds__(128) k_adj_predict(AdjArgs A) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < A.L.n && s < activeCount(A)) adjPredictSlot(A, s);
}

// Predict's pair terms of slot s gathered by a group of G lanes over the perception disk (every lane takes part);
// lane 0 writes the state adjoint before the step and the radius gradient. valid: s is active at the step.
template <int G>
__device__ void adjGatherSlot(const AdjArgs& A, int s, int lane, bool valid) {
    const SwarmParams& P = A.P;
    const VenueArgs& V = A.V;
    const TapeLayout& L = A.L;
    const float4* pos = A.f4 + L.pos0();
    const float4* pred = A.f4 + L.pred();
    constexpr int MAXR = 2 * 4 + 1;   // perc_ring <= 4
    uint32_t rk0[MAXR], len[MAXR];
    uint32_t total = 0;
    float4 p = make_float4(0.0f, 0.0f, 0.0f, 0.0f), ls = p;
    float ri = 0.0f;
    uint32_t id = 0;
    const int R = P.perc_ring;
#pragma unroll
    for (int j = 0; j < MAXR; ++j) { rk0[j] = 0u; len[j] = 0u; }
    if (valid) {
        id = A.sid[s];
        p = pos[s];
        ri = A.prm[s].x;
        ls = A.lamSep[s];
        const uint32_t cid = A.skey[s];
        const int resX = V.resX, resY = V.resY;
        const int cx = int(cid % uint32_t(resX)), cy = int(cid / uint32_t(resX));
        // each row's cells that can hold an agent within the reach (cells widened by margin, as predict trims)
        const float csx = V.dspanX / float(resX), csy = V.dspanY / float(resY);
        const float margin = 0.01f * smax(csx, csy);
        const float rr = smin(sqrtf(P.r_perc2), A.gatherReach) + margin;
#pragma unroll
        for (int j = 0; j < MAXR; ++j) {
            const int ny = cy - R + j;
            if (j > 2 * R || ny < 0 || ny >= resY) continue;
            const float ylo = V.dminY + float(ny) * csy - margin, yhi = V.dminY + float(ny + 1) * csy + margin;
            const float dy = fmaxf(0.0f, fmaxf(ylo - p.y, p.y - yhi));
            if (dy >= rr) continue;
            const float w = sqrtf(rr * rr - dy * dy) + margin;
            const int xlo = max(max(cx - R, 0), int(floorf((p.x - w - V.dminX) / csx)));
            const int xhi = min(min(cx + R, resX - 1), int(floorf((p.x + w - V.dminX) / csx)));
            if (xlo > xhi) continue;
            rk0[j] = A.start[xlo + ny * resX];
            len[j] = A.start[xhi + 1 + ny * resX] - rk0[j];
            total += len[j];
        }
    }
    f3 lp{0.0f, 0.0f, 0.0f};
    float lr = 0.0f;
    for (uint32_t idx = uint32_t(lane); idx < total; idx += uint32_t(G)) {
        uint32_t k = idx, j = 0;
        while (k >= len[j]) { k -= len[j]; ++j; }
        k += rk0[j];
        if (int(k) == s) continue;
        const float4 op = pos[k];
        const f3 o = xyz(p) - xyz(op);
        const float dxy2 = dot(xy(o), xy(o));
        if (!(dxy2 < P.r_perc2)) continue;
        const float4 lk = A.lamSep[k];
        const float dc = ri + A.prm[k].x;
        const float rs = dc + P.sep_margin, rs2 = rs * rs;
        const float d2 = dot(o, o);
        if (d2 < rs2) {   // separation f = k_sep w^2 dir, w = 1 - |o| / rs: F^T (lambda_s - lambda_k)
            const f2 dl{ls.x - lk.x, ls.y - lk.y};
            const float D = sqrtf(d2);
            const float w = 1.0f - D / rs;
            const bool stacked = dxy2 <= P.stacked_xy2;
            float rxy = 0.0f;
            f2 dir;
            if (stacked) dir = pairDirection(id, A.sid[k], P.hash_to_radians);
            else { rxy = sqrtf(dxy2); dir = xy(o) / rxy; }
            const float kd = dot(dir, dl);
            if (D > 0.0f) {
                const float c1 = -2.0f * P.k_sep * w / (D * rs) * kd;
                lp = lp + o * c1;
            }
            if (!stacked) {
                const float c2 = P.k_sep * w * w / rxy;
                lp.x += c2 * (dl.x - dir.x * kd);
                lp.y += c2 * (dl.y - dir.y * kd);
            }
            lr += 2.0f * P.k_sep * w * D / rs2 * kd;
        }
        if (__float_as_int(pred[k].w) == s && lk.z != 0.0f) {   // this slot is k's nearest agent ahead
            const float dxy = sqrtf(dxy2);
            if (dxy > 0.0f) { lp.x += o.x / dxy * lk.z; lp.y += o.y / dxy * lk.z; }
            lr -= lk.z;
        }
    }
    lp.x = groupSum<G>(lp.x);
    lp.y = groupSum<G>(lp.y);
    lp.z = groupSum<G>(lp.z);
    lr = groupSum<G>(lr);
    if (!valid || lane != 0) return;
    const float4 lp4 = A.lamP[s];
    const float4 lv = A.lamV[s];
    A.lamOut[2 * size_t(id)] = make_float4(lp.x + lp4.x, lp.y + lp4.y, lp.z + lp4.z, 0.0f);
    A.lamOut[2 * size_t(id) + 1] = make_float4(lv.x, lv.y, lv.z, 0.0f);
    A.gR[id] += double(A.lamR[s] + lr);
}

__global__ void __launch_bounds__(128) k_adj_gather(AdjArgs A) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    adjGatherSlot<1>(A, s, 0, s < A.L.n && s < activeCount(A));
}

// ---- the whole reverse step as one persistent kernel ----
// Every block stays resident (a cooperative launch); the phases are separated by a grid barrier on one word: block 0
// adds 2^31 - (blocks - 1), every other block 1, so the word's top bit flips once all have arrived; a block waits for
// the flip at most ADJ_BARRIER_WAIT_NS of %globaltimer, then records ERR_TIMEOUT and leaves the kernel, as does every
// waiting block that finds ERR_TIMEOUT set (the host reports SWARM_E_TIMEOUT). Only the last arrival's add flips the
// bit: that block goes on without polling (its add acquires), and nothing is read before the add.
constexpr uint64_t ADJ_BARRIER_WAIT_NS = 1000000000ull;

__device__ __forceinline__ uint64_t adjNs() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Returns false (the same in every thread of the block) when the block must leave the kernel: its wait ran out, or
// another block's did (no phase runs on data another block has not finished)
__device__ __forceinline__ bool adjBarrier(const AdjArgs& A) {
    __shared__ int leave;
    __syncthreads();
    if (threadIdx.x == 0) {
        cuda::atomic_ref<unsigned, cuda::thread_scope_device> word(*A.barrier);
        const unsigned add = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1u) : 1u;
        const unsigned old = word.fetch_add(add, cuda::memory_order_acq_rel);
        int out = 0;
        if ((((old + add) ^ old) & 0x80000000u) == 0u) {
            cuda::atomic_ref<int, cuda::thread_scope_device> err(*A.err);
            const uint64_t t0 = adjNs();
            unsigned polls = 0;
            while (((word.load(cuda::memory_order_acquire) ^ old) & 0x80000000u) == 0u) {
                if (adjNs() - t0 > ADJ_BARRIER_WAIT_NS) { err.fetch_or(ERR_TIMEOUT, cuda::memory_order_relaxed); out = 1; break; }
                if (++polls % 64u == 0u && (err.load(cuda::memory_order_relaxed) & ERR_TIMEOUT)) { out = 1; break; }
            }
        }
        leave = out;
    }
    __syncthreads();
    return leave == 0;
}

// Timing on: block 0 adds the span since *t0 to stamps[i] and restarts the clock
__device__ __forceinline__ void adjStamp(const AdjArgs& A, int i, uint64_t& t0) {
    if (A.stamps && blockIdx.x == 0 && threadIdx.x == 0) {
        const uint64_t t = adjNs();
        A.stamps[i] += t - t0;
        t0 = t;
    }
}

template <int G>
__global__ void __launch_bounds__(ADJ_FUSED_THREADS, 1) k_adj_step_fused(AdjArgs A) {
    __shared__ double warpSum[ADJ_FUSED_THREADS / 32];
    const int n = A.L.n, K = A.L.K;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    const int lane = int(threadIdx.x) % G;
    uint64_t t0 = A.stamps ? adjNs() : 0;
    // final pass (and the loss sum of the block's slots)
    double d = 0.0;
    for (int s = tid; s < n; s += stride) d += adjFinalSlot(A, s);
    const double t = blockSum<ADJ_FUSED_THREADS>(d, warpSum);
    if (threadIdx.x == 0) A.lossPart[blockIdx.x] = t;
    if (!adjBarrier(A)) return;
    adjStamp(A, 0, t0);
    // the sweeps, last to first: G lanes per slot (warp-uniform loop)
    const int groups = stride / G, g0 = tid / G;
    const int nActive = activeCount(A);
    if (nActive <= groups) {   // one slot per lane group: its rows and status once for all the sweeps
        const int s = g0;
        const bool valid = sweepsSlot(A, s);
        uint32_t rows[6] = {0u, 0u, 0u, 0u, 0u, 0u};
        if (valid) rows3(A, A.skey[s], rows, rows + 3);
        for (int k = K; k >= 1; --k) {
            if (g0 - (g0 % (32 / G)) < nActive) adjSweepSlot<G>(A, s, lane, valid, k, rows);
            if (!adjBarrier(A)) return;
        }
    } else {
        for (int k = K; k >= 1; --k) {
            for (int base = g0 - (g0 % (32 / G)); base < nActive; base += groups) {
                const int s = base + (g0 % (32 / G));
                adjSweepSlot<G>(A, s, lane, sweepsSlot(A, s), k);
            }
            if (!adjBarrier(A)) return;
        }
    }
    adjStamp(A, 1, t0);
    for (int s = tid; s < nActive; s += stride) adjPredictSlot(A, s);
    if (!adjBarrier(A)) return;
    adjStamp(A, 2, t0);
    if (A.stamps && blockIdx.x == 0 && threadIdx.x == 0) A.stamps[4] = t0;   // the gather's start
    for (int base = g0 - (g0 % (32 / G)); base < nActive; base += groups) {
        const int s = base + (g0 % (32 / G));
        adjGatherSlot<G>(A, s, lane, s < nActive);
    }
    if (A.stamps) {   // the gather ends when the last block leaves
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            cuda::atomic_ref<unsigned, cuda::thread_scope_device> done(A.barrier[1]);
            if (done.fetch_add(1u, cuda::memory_order_acq_rel) == gridDim.x - 1) {
                A.stamps[3] += adjNs() - A.stamps[4];
                done.store(0u, cuda::memory_order_relaxed);
            }
        }
    }
}

inline int blocksOf(int n, int t) { return (n + t - 1) / t; }

}  // namespace

void launch_adjoint_step(AdjArgs& A, cudaStream_t st, int64_t* launches) {
    const int n = A.L.n;
    k_adj_final<<<adjFinalBlocks(n), ADJ_FINAL_THREADS, 0, st>>>(A);
    for (int k = A.L.K; k >= 1; --k) {
        A.sweep = k;
        k_adj_sweep<<<blocksOf(n, 128), 128, 0, st>>>(A);
    }
    k_adj_predict<<<blocksOf(n, 128), 128, 0, st>>>(A);
    k_adj_gather<<<blocksOf(n, 128), 128, 0, st>>>(A);
    *launches += 3 + A.L.K;
}

namespace {
// SM count and resident blocks of the fused reverse, per host thread and device ordinal
constexpr int ADJ_MAX_DEVICES = 64;
thread_local int g_smsOf[ADJ_MAX_DEVICES], g_perSmOf[ADJ_MAX_DEVICES];
thread_local int g_sms = 0, g_perSm = 0;
void fusedConfig() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= ADJ_MAX_DEVICES) dev = 0;
    if (!g_smsOf[dev]) {
        int sms = 0, perSm = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k_adj_step_fused<ADJ_LANES>, ADJ_FUSED_THREADS, 0) == cudaSuccess) {
            g_smsOf[dev] = sms;
            g_perSmOf[dev] = perSm;
        }
    }
    g_sms = g_smsOf[dev] > 0 ? g_smsOf[dev] : 1;
    g_perSm = g_perSmOf[dev];
}
}  // namespace

// The fused reverse's block: the state's lane groups spread over every SM (threads = n x lanes / SMs rounded up to a
// warp, 128..512), one block per SM; larger states take several slots per lane group
int adjFusedThreads(int n) {
    fusedConfig();
    const int64_t lanes = int64_t(n) * ADJ_LANES;
    int t = int((lanes + g_sms - 1) / g_sms);
    t = (t + 31) / 32 * 32;
    return std::max(128, std::min(t, ADJ_FUSED_THREADS));
}

int adjFusedBlocks(int n) {
    fusedConfig();
    const int resident = g_sms * g_perSm;
    const int threads = adjFusedThreads(n);
    const int want = int((int64_t(n) * ADJ_LANES + threads - 1) / threads);
    return std::max(1, std::min(want, resident));
}

cudaError_t launch_adjoint_step_fused(AdjArgs& A, cudaStream_t st) {
    fusedConfig();
    if (g_sms * g_perSm <= 0) return cudaErrorCooperativeLaunchTooLarge;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(adjFusedBlocks(A.L.n)));
    cfg.blockDim = dim3(unsigned(adjFusedThreads(A.L.n)));
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_adj_step_fused<ADJ_LANES>, A);
}

}  // namespace swarm_gpu
