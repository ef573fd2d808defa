// Plan venues on grids (SI units, per-agent radius): the static contacts follow the reference's analytic-venue
// branch (DedovSergei/swarm-crowd-simulation src/cpu_crowd_sim.cpp: floorUnderReach :291-297, clearWalls :386-399,
// wallPlaneProbe :444-447, resolveStatic :483-514) with the wall query answered by a horizontal wall SDF grid, and
// e_goal = -grad D / |grad D| of a geodesic distance grid in place of the reference's navigation field lookup.
#pragma once

#include "device_math.cuh"
#include "step_args.cuh"

namespace swarm_gpu {

struct GridVenue {
    const SwarmParams& P;
    const VenueArgs& V;

    // The wall query: (direction away from the nearest wall, its distance); distance WALL_NONE when it is at least
    // `reach` or p lies outside the field. Bilinear value and gradient of the wall SDF.
    __device__ f3 wall(f2 p, float reach) const {
        const float fx = (p.x - V.wox) * V.winv, fy = (p.y - V.woy) * V.winv;
        if (!(fx >= 0.0f && fy >= 0.0f && fx <= float(V.wnx - 1) && fy <= float(V.wny - 1))) return f3{0.0f, 0.0f, WALL_NONE};
        const int ix = smin(int(floorf(fx)), V.wnx - 2), iy = smin(int(floorf(fy)), V.wny - 2);
        const float wx = fx - float(ix), wy = fy - float(iy);
        const size_t r0 = size_t(iy) * size_t(V.wnx) + size_t(ix), r1 = r0 + size_t(V.wnx);
        float c00, c10, c01, c11;
        if (V.wallFloor) {
            c00 = __ldg(V.wallFloor + r0).x; c10 = __ldg(V.wallFloor + r0 + 1).x;
            c01 = __ldg(V.wallFloor + r1).x; c11 = __ldg(V.wallFloor + r1 + 1).x;
        } else {
            c00 = __ldg(V.wall + r0); c10 = __ldg(V.wall + r0 + 1); c01 = __ldg(V.wall + r1); c11 = __ldg(V.wall + r1 + 1);
        }
        const float d = mix(mix(c00, c10, wx), mix(c01, c11, wx), wy);
        if (d >= reach) return f3{0.0f, 0.0f, WALL_NONE};
        f2 g{mix(c10 - c00, c11 - c01, wy) * V.winv, mix(c01 - c00, c11 - c10, wx) * V.winv};
        f2 n = safeNormalize(g, P.safe_eps);
        return f3{n.x, n.y, d};
    }
    __device__ __forceinline__ float wallDist(f2 p) const { return wall(p, WALL_NONE).z; }
    __device__ __forceinline__ size_t floorNode(f2 p) const {
        const float fx = (p.x - V.wox) * V.winv + 0.5f, fy = (p.y - V.woy) * V.winv + 0.5f;
        const int ix = sclamp(int(floorf(fx)), 0, V.wnx - 1), iy = sclamp(int(floorf(fy)), 0, V.wny - 1);
        return size_t(iy) * size_t(V.wnx) + size_t(ix);
    }
    __device__ __forceinline__ float floorHeight(f2 p) const {
        if (V.wallFloor) return __ldg(V.wallFloor + floorNode(p)).y;
        return V.floorH ? __ldg(V.floorH + floorNode(p)) : 0.0f;
    }
    __device__ __forceinline__ float speedFactor(f3 p) const { return V.speedF ? __ldg(V.speedF + floorNode(xy(p))) : 1.0f; }
    __device__ __forceinline__ float map(f3 p) const { return smin(wallDist(xy(p)), p.z - floorHeight(xy(p))); }

    // e_goal = -grad D / |grad D| of the bilinear interpolant of the distance grid (the nearest exit's, or D = one
    // exit's own field on the same grid)
    __device__ __forceinline__ f2 goal(f3 p) const { return goalIn(V.nav, p); }
    __device__ f2 goalIn(const float* D, f3 p) const {
        float fx = (p.x - V.nox) * V.ninv, fy = (p.y - V.noy) * V.ninv;
        fx = sclamp(fx, 0.0f, float(V.nnx - 1));
        fy = sclamp(fy, 0.0f, float(V.nny - 1));
        const int ix = smin(int(floorf(fx)), V.nnx - 2), iy = smin(int(floorf(fy)), V.nny - 2);
        const float wx = fx - float(ix), wy = fy - float(iy);
        const size_t r0 = size_t(iy) * size_t(V.nnx) + size_t(ix), r1 = r0 + size_t(V.nnx);
        const float d00 = __ldg(D + r0), d10 = __ldg(D + r0 + 1), d01 = __ldg(D + r1), d11 = __ldg(D + r1 + 1);
        f2 g{mix(d10 - d00, d11 - d01, wy), mix(d01 - d00, d11 - d10, wx)};
        return safeNormalize(f2{-g.x, -g.y}, P.safe_eps);
    }

    __device__ __forceinline__ bool exits(float4 p) const {
        const bool outDomain = p.x < V.dminX || p.x > V.dmaxX || p.y < V.dminY || p.y > V.dmaxY;
        if (V.exitMask) {   // the exit mask: the nav node nearest to p
            const float fx = (p.x - V.nox) * V.ninv + 0.5f, fy = (p.y - V.noy) * V.ninv + 0.5f;
            const int ix = sclamp(int(floorf(fx)), 0, V.nnx - 1), iy = sclamp(int(floorf(fy)), 0, V.nny - 1);
            return outDomain || __ldg(V.exitMask + size_t(iy) * size_t(V.nnx) + size_t(ix)) != 0;
        }
        const bool out = p.x < V.exloX || p.x > V.exhiX || p.y < V.exloY || p.y > V.exhiY;
        return (out && p.z < V.exMaxZ) || outDomain;
    }

    __device__ __forceinline__ bool floorUnderReach(f3 c, float zFrom, float down, float r, float& zFloor) const {
        const float h = floorHeight(xy(c));
        zFloor = h;
        if (c.z <= h) return h <= smax(zFrom, c.z) + r;
        return h >= c.z - down;
    }
    __device__ __forceinline__ bool restOnFloor(f3& np, f3& nv, float zFrom, float r) const {
        float zFloor;
        if (floorUnderReach(np, zFrom, r, r, zFloor) && np.z < zFloor + r) { np.z = zFloor + r; nv.z = 0.0f; return true; }
        return false;
    }
    __device__ __forceinline__ bool settleOnFloor(f3& np, f3& nv, float zFrom, float r) const {
        float zFloor;
        if (floorUnderReach(np, zFrom, P.floor_settle_reach, r, zFloor)) { np.z = zFloor + r; nv.z = 0.0f; return true; }
        return false;
    }
    __device__ bool clearWalls(f3& np, f3& nv, f3& wallOut, float r) const {
        bool moved = false;
        wallOut = f3{0.0f, 0.0f, 0.0f};
        for (int pass = 0; pass < P.wall_passes; ++pass) {
            const f3 w = wall(xy(np), P.feeler_reach);
            if (w.z >= r) {
                if (w.z < WALL_NONE) wallOut = f3{w.x, w.y, w.z - r};
                break;
            }
            setXY(np, xy(np) + f2{w.x, w.y} * (r - w.z));
            moved = true;
            wallOut = f3{w.x, w.y, 0.0f};
            const float vDotN = dot(xy(nv), f2{w.x, w.y});
            if (vDotN < 0.0f) setXY(nv, xy(nv) - f2{w.x, w.y} * vDotN);
        }
        return moved;
    }
    __device__ f3 wallPlaneProbe(f3 np, float r) const {
        const f3 w = wall(xy(np), P.plane_probe_reach);
        return w.z >= 0.0f && w.z < WALL_NONE ? f3{w.x, w.y, smax(w.z - r, 0.0f)} : f3{0.0f, 0.0f, 0.0f};
    }
    __device__ __forceinline__ bool solid(f3 p) const { return map(p) <= 0.0f; }
    __device__ bool sweepBack(f3 pOld, f3& np, f3& nv) const {
        if (!solid(np)) return false;
        float lo = 0.0f, hi = 1.0f;
        if (!solid(f3{np.x, np.y, pOld.z})) lo = 1.0f;
        for (int i = 0; i < P.sweep_bisections; ++i) {
            float t = 0.5f * (lo + hi);
            f2 m = mix(xy(pOld), xy(np), t);
            if (solid(f3{m.x, m.y, pOld.z})) hi = t;
            else lo = t;
        }
        f2 d = safeNormalize(xy(np) - xy(pOld), P.safe_eps);
        f2 m = mix(xy(pOld), xy(np), lo);
        np = f3{m.x, m.y, pOld.z};
        float vd = dot(xy(nv), d);
        if (vd > 0.0f) setXY(nv, xy(nv) - d * vd);
        nv.z = 0.0f;
        return true;
    }
    __device__ bool resolveStatic(f3 pOld, f3& np, f3& nv, bool settle, f3& wallOut, uint32_t& contact, float r) const {
        bool grounded = settle ? settleOnFloor(np, nv, pOld.z, r) : restOnFloor(np, nv, pOld.z, r);
        if (!grounded && sweepBack(pOld, np, nv)) {
            contact |= C_SWEEP;
            grounded = restOnFloor(np, nv, pOld.z, r);
        }
        if (grounded) contact |= C_FLOOR;
        const bool walls = clearWalls(np, nv, wallOut, r);
        if (walls) {
            contact |= C_WALL;
            if (grounded) {
                if (settleOnFloor(np, nv, pOld.z, r)) contact |= C_FLOOR;
                f3 w2;
                const bool again = clearWalls(np, nv, w2, r);
                if (w2.x != 0.0f || w2.y != 0.0f) wallOut = w2;
                if (again && restOnFloor(np, nv, pOld.z, r)) contact |= C_FLOOR;
            } else if (restOnFloor(np, nv, pOld.z, r)) {
                contact |= C_FLOOR;
            }
        }
        return grounded;
    }
    // The step-up limit over the floor heightfield (the reference's limitStepUp, cpu_crowd_sim.cpp:566-591, baked
    // branch, with the floor grid in place of the baked column scan). The floor is the nearest node's height: level
    // treads with vertical risers, the reference's "exact venue", where a floor in the window (f0 + tol, f0 + max]
    // is never wall-steep and the window's top decides (rule (a), stepUpBlocked :531-533): a move is blocked when
    // the floor under its end lies more than max_step_up above f0. No floor grid: a flat floor, never blocked.
    __device__ __forceinline__ int stepUpWindow(f2 p, float f0) const {   // 0 level or lower, 1 in the window, 2 above
        const float h = floorHeight(p);
        if (h > f0 + P.max_step_up) return 2;
        return h > f0 + P.step_up_tol ? 1 : 0;
    }
    // The riser's normal at p: the floor's central differences over the neighbouring nodes, pointing out of the
    // higher column (the reference's face normal, the solid's gradient)
    __device__ f2 stepUpFace(f2 p) const {
        const float fx = (p.x - V.wox) * V.winv + 0.5f, fy = (p.y - V.woy) * V.winv + 0.5f;
        const int ix = sclamp(int(floorf(fx)), 0, V.wnx - 1), iy = sclamp(int(floorf(fy)), 0, V.wny - 1);
        const int x0 = smax(ix - 1, 0), x1 = smin(ix + 1, V.wnx - 1), y0 = smax(iy - 1, 0), y1 = smin(iy + 1, V.wny - 1);
        const size_t row = size_t(iy) * size_t(V.wnx);
        const f2 g{__ldg(V.floorH + row + size_t(x0)) - __ldg(V.floorH + row + size_t(x1)),
                   __ldg(V.floorH + size_t(y0) * size_t(V.wnx) + size_t(ix)) - __ldg(V.floorH + size_t(y1) * size_t(V.wnx) + size_t(ix))};
        return safeNormalize(g, P.safe_eps);
    }
    // stepUpScan (cpu_crowd_sim.cpp:539-563): only the end can block (rule (a)); the last allowed sample before it
    // starts the bisection
    __device__ float stepUpScan(f2 p0, f2 p1, float f0, f2& n) const {
        n = f2{0.0f, 0.0f};
        const float len = length(p1 - p0);
        const int ns = sclamp(int(ceilf(len / P.step_up_sample)), 1, P.step_up_max_samples);
        const f2 pe = mix(p0, p1, float(ns) / float(ns));
        if (stepUpWindow(pe, f0) != 2) return 1.0f;
        n = stepUpFace(pe);
        int lastOk = 0;
        for (int i = 1; i < ns; ++i)
            if (stepUpWindow(mix(p0, p1, float(i) / float(ns)), f0) != 2) lastOk = i;
        float lo = float(lastOk) / float(ns), hi = float(lastOk + 1) / float(ns);
        for (int i = 0; i < P.step_up_bisections; ++i) {
            const float t = 0.5f * (lo + hi);
            const f2 q = mix(p0, p1, t);
            if (stepUpWindow(q, f0) == 2) { hi = t; n = stepUpFace(q); }
            else lo = t;
        }
        return lo;
    }
    // limitStepUp (cpu_crowd_sim.cpp:566-591): back to the riser, the rest of the move along it (veering off by the
    // slide angles until a slide is allowed), the velocity into it removed, settled from the start-of-step height.
    // Radius r: the agent's own (the floor contact of every grid-venue query).
    __device__ bool limitStepUp(f3 pOld, f3& np, f3& nv, float r) const {
        if (!V.floorH) return false;
        float f0;
        if (!floorUnderReach(pOld, pOld.z, P.step_up_floor_reach, r, f0)) f0 = pOld.z - P.step_up_floor_reach;
        f2 n;
        const float t = stepUpScan(xy(pOld), xy(np), f0, n);
        if (t >= 1.0f) return false;
        f2 q = mix(xy(pOld), xy(np), t);
        const f2 rest = xy(np) - q;
        const f2 tangent = rest - n * dot(rest, n);
        const float lt = length(tangent);
        if (lt > 0.0f) {
            for (int k = 0; k < P.step_up_slide_tries; ++k) {
                const f2 slide = q + tangent * P.step_up_slide[k][0] + n * (lt * P.step_up_slide[k][1]);
                f2 n2;
                if (stepUpScan(q, slide, f0, n2) >= 1.0f) { q = slide; break; }
            }
        }
        const float vn = dot(xy(nv), n);
        if (vn < 0.0f) setXY(nv, xy(nv) - n * vn);
        float zFloor;
        if (floorUnderReach(f3{q.x, q.y, pOld.z}, pOld.z, P.floor_settle_reach, r, zFloor)) {
            np = f3{q.x, q.y, zFloor + r};
            nv.z = 0.0f;
        } else {
            np = f3{q.x, q.y, smin(np.z, pOld.z)};
        }
        return true;
    }
    __device__ f3 calcGradient(f3 p) const {
        const f3 kxyy{1.0f, -1.0f, -1.0f}, kyyx{-1.0f, -1.0f, 1.0f}, kyxy{-1.0f, 1.0f, -1.0f}, kxxx{1.0f, 1.0f, 1.0f};
        const float h = P.obstacle_grad_h;
        f3 a = kxyy * map(p + kxyy * h), b = kyyx * map(p + kyyx * h), c = kyxy * map(p + kyxy * h), d = kxxx * map(p + kxxx * h);
        return (a + b + c + d) * P.obstacle_grad_scale;
    }
    __device__ __forceinline__ float sceneDist(f3 p, bool& onFence) const { onFence = false; return map(p); }
    __device__ __forceinline__ f2 sceneNormal(f3 p, bool) const { return xy(safeNormalize(calcGradient(p), P.safe_eps)); }
    __device__ __forceinline__ void fenceProject(f3&) const {}
};

}  // namespace swarm_gpu
