// The reference's baked terrace on the GPU: stadium.sdf sampled with exact float weights (never the texture unit's
// 8-bit filter weights), the analytic pitch fence, the egress router, and the static contacts and step-up limit that
// read them. Restated from DedovSergei/swarm-crowd-simulation src/cpu_crowd_sim.cpp and src/sdf.cpp (the CPU port of
// shaders/physics.comp); each function cites its lines there.
#pragma once

#include "device_math.cuh"
#include "step_args.cuh"

namespace swarm_gpu {

struct Stadium {
    const SwarmParams& P;
    const VenueArgs& V;

    __device__ __forceinline__ float texel(int x, int y, int z) const {
        return __ldg(V.sdf + (size_t(x) * size_t(V.sdfRes) + size_t(y)) * size_t(V.sdfRes) + size_t(z));
    }
    __device__ __forceinline__ f3 toTex(f3 p) const {   // 1 + (p - SDF_MIN) * (1 / SDF_SPACING)
        return {1.0f + (p.x - V.sdfMinX) * V.sdfInv, 1.0f + (p.y - V.sdfMinY) * V.sdfInv, 1.0f + (p.z - V.sdfMinZ) * V.sdfInv};
    }

    // src/sdf.cpp:21-43 sampleSDF
    __device__ float map(f3 pos) const {
        const int res = V.sdfRes;
        const float fr = float(res);
        f3 uvw{(1.5f + (pos.x - V.sdfMinX) / V.sdfSpacing) / fr, (1.5f + (pos.y - V.sdfMinY) / V.sdfSpacing) / fr,
               (1.5f + (pos.z - V.sdfMinZ) / V.sdfSpacing) / fr};
        if (uvw.x < 0.0f || uvw.y < 0.0f || uvw.z < 0.0f || uvw.x > 1.0f || uvw.y > 1.0f || uvw.z > 1.0f) return 1.0f;
        f3 t{uvw.x * fr - 0.5f, uvw.y * fr - 0.5f, uvw.z * fr - 0.5f};
        f3 base{floorf(t.x), floorf(t.y), floorf(t.z)};
        f3 f{t.x - base.x, t.y - base.y, t.z - base.z};
        const int x0 = int(base.x), y0 = int(base.y), z0 = int(base.z);
        const int xa = sclamp(x0, 0, res - 1), xb = sclamp(x0 + 1, 0, res - 1);
        const int ya = sclamp(y0, 0, res - 1), yb = sclamp(y0 + 1, 0, res - 1);
        const int za = sclamp(z0, 0, res - 1), zb = sclamp(z0 + 1, 0, res - 1);
        float c00 = mix(texel(xa, ya, za), texel(xb, ya, za), f.x);
        float c10 = mix(texel(xa, yb, za), texel(xb, yb, za), f.x);
        float c01 = mix(texel(xa, ya, zb), texel(xb, ya, zb), f.x);
        float c11 = mix(texel(xa, yb, zb), texel(xb, yb, zb), f.x);
        return mix(mix(c00, c10, f.y), mix(c01, c11, f.y), f.z);
    }

    // cpu_crowd_sim.cpp:255-261
    __device__ __forceinline__ float columnLevel(int i0x, int i0y, f2 w, int k) const {
        k = sclamp(k, 0, V.sdfRes - 1);
        float c0 = mix(texel(i0x, i0y, k), texel(i0x + 1, i0y, k), w.x);
        float c1 = mix(texel(i0x, i0y + 1, k), texel(i0x + 1, i0y + 1, k), w.x);
        return mix(c0, c1, w.y);
    }

    // cpu_crowd_sim.cpp:263-287 mapExactGrad: (gradient, value)
    __device__ float4 mapExactGrad(f3 p) const {
        const int res = V.sdfRes;
        f3 f = toTex(p);
        const float hiLim = float(res) - 0.5f;
        const bool outside = f.x < -0.5f || f.y < -0.5f || f.z < -0.5f || f.x > hiLim || f.y > hiLim || f.z > hiLim;
        if (outside) return make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        const int ix = sclamp(int(floorf(f.x)), 0, res - 2), iy = sclamp(int(floorf(f.y)), 0, res - 2),
                  iz = sclamp(int(floorf(f.z)), 0, res - 2);
        f3 w{f.x - float(ix), f.y - float(iy), f.z - float(iz)};
        float c000 = texel(ix, iy, iz), c100 = texel(ix + 1, iy, iz), c010 = texel(ix, iy + 1, iz), c110 = texel(ix + 1, iy + 1, iz);
        float c001 = texel(ix, iy, iz + 1), c101 = texel(ix + 1, iy, iz + 1), c011 = texel(ix, iy + 1, iz + 1);
        float c111 = texel(ix + 1, iy + 1, iz + 1);
        float x00 = mix(c000, c100, w.x), x10 = mix(c010, c110, w.x);
        float x01 = mix(c001, c101, w.x), x11 = mix(c011, c111, w.x);
        float y0 = mix(x00, x10, w.y), y1 = mix(x01, x11, w.y);
        float gx = mix(mix(c100 - c000, c110 - c010, w.y), mix(c101 - c001, c111 - c011, w.y), w.z);
        float gy = mix(x10 - x00, x11 - x01, w.z);
        float gz = y1 - y0;
        return make_float4(gx * V.sdfInv, gy * V.sdfInv, gz * V.sdfInv, mix(y0, y1, w.z));
    }

    // cpu_crowd_sim.cpp:289-316 floorUnderReach
    __device__ bool floorUnderReach(f3 c, float zFrom, float down, float& zFloor) const {
        const int res = V.sdfRes;
        zFloor = 0.0f;
        f3 f = toTex(c);
        const float hiLim = float(res) - 1.0f;
        if (f.x < 0.0f || f.y < 0.0f || f.x > hiLim || f.y > hiLim) return false;
        const int i0x = smin(int(floorf(f.x)), res - 2), i0y = smin(int(floorf(f.y)), res - 2);
        f2 w{f.x - float(i0x), f.y - float(i0y)};
        int k = int(floorf(f.z));
        float vLo = columnLevel(i0x, i0y, w, k), vHi = columnLevel(i0x, i0y, w, k + 1);
        const bool inSolid = mix(vLo, vHi, f.z - float(k)) <= 0.0f;
        const float fLimit = f.z + (inSolid ? smax(zFrom, c.z) + P.body_radius - c.z : -down) * V.sdfInv;
        for (int cell = 0; cell < P.floor_search_cells; ++cell) {
            float fEnd = inSolid ? smin(float(k + 1), fLimit) : smax(float(k), fLimit);
            float vEnd = mix(vLo, vHi, fEnd - float(k));
            if (inSolid ? vEnd > 0.0f : vEnd <= 0.0f) {
                float fRoot = float(k) + vLo / (vLo - vHi);
                zFloor = V.sdfMinZ + (fRoot - 1.0f) / V.sdfInv;
                return true;
            }
            if (fEnd == fLimit) return false;
            if (inSolid) { ++k; vLo = vHi; vHi = columnLevel(i0x, i0y, w, k + 1); }
            else         { --k; vHi = vLo; vLo = columnLevel(i0x, i0y, w, k); }
        }
        return false;
    }

    // src/sdf.cpp:45-57, 64-82: the pitch fence
    __device__ __forceinline__ static float sdBox2(f2 p, f2 half) {
        f2 q{fabsf(p.x) - half.x, fabsf(p.y) - half.y};
        f2 qp{smax(q.x, 0.0f), smax(q.y, 0.0f)};
        return length(qp) + smin(smax(q.x, q.y), 0.0f);
    }
    __device__ __forceinline__ static f2 sdBox2Grad(f2 p, f2 half) {
        f2 q{fabsf(p.x) - half.x, fabsf(p.y) - half.y};
        f2 s{p.x < 0.0f ? -1.0f : 1.0f, p.y < 0.0f ? -1.0f : 1.0f};
        f2 g;
        if (smax(q.x, q.y) > 0.0f) {
            f2 qp{smax(q.x, 0.0f), smax(q.y, 0.0f)};
            g = qp / length(qp);
        } else {
            g = q.x > q.y ? f2{1.0f, 0.0f} : f2{0.0f, 1.0f};
        }
        return s * g;
    }
    __device__ __forceinline__ f2 fenceC() const { return {P.fence_center[0], P.fence_center[1]}; }
    __device__ __forceinline__ f2 fenceMid() const { return {P.fence_half_mid[0], P.fence_half_mid[1]}; }
    __device__ __forceinline__ float sdFence(f3 p) const { return fabsf(sdBox2(xy(p) - fenceC(), fenceMid())) - P.fence_half_thk_coll; }
    __device__ __forceinline__ f2 sdFenceGradient(f3 p) const {
        f2 rel = xy(p) - fenceC();
        float box = sdBox2(rel, fenceMid());
        return (box < 0.0f ? -1.0f : 1.0f) * sdBox2Grad(rel, fenceMid());
    }

    // cpu_crowd_sim.cpp:99-116 fenceCCD
    __device__ bool fenceCCD(f3 pOld, f3& pNew, f3& vel) const {
        float sOld = sdBox2(xy(pOld) - fenceC(), fenceMid());
        float sNew = sdBox2(xy(pNew) - fenceC(), fenceMid());
        if (sOld * sNew >= 0.0f) return false;
        float side = sOld > 0.0f ? 1.0f : -1.0f;
        float lo = 0.0f;
        if (side * sOld > P.fence_half_thk_coll) {
            float hi = 1.0f;
            for (int i = 0; i < P.fence_ccd_bisections; ++i) {
                float t = 0.5f * (lo + hi);
                if (side * sdBox2(mix(xy(pOld), xy(pNew), t) - fenceC(), fenceMid()) > P.fence_half_thk_coll) lo = t;
                else hi = t;
            }
        }
        setXY(pNew, mix(xy(pOld), xy(pNew), lo));
        f2 n = sdFenceGradient(pNew);
        float vn = dot(xy(vel), n);
        if (vn < 0.0f) setXY(vel, xy(vel) - n * vn);
        return true;
    }

    // cpu_crowd_sim.cpp:154-172 egressTarget / egressDirection
    __device__ f2 goal(f3 p) const {
        f2 s{p.x < 0.0f ? -1.0f : 1.0f, p.y < 0.0f ? -1.0f : 1.0f};
        f2 a{fabsf(p.x), fabsf(p.y)};
        const bool alongX = a.y >= a.x;
        const float lat = alongX ? a.x : a.y;
        const float dep = alongX ? a.y : a.x;
        f2 t;
        if (lat < P.avenue_half && dep >= P.walkway_min) t = {0.0f, P.avenue_target_depth};
        else if (dep >= P.walkway_min && dep < P.walkway_max) t = {0.0f, P.walkway_centre};
        else if (dep >= P.walkway_max && lat < P.aisle_max) t = {P.aisle_centre, P.walkway_centre};
        else if (dep >= P.walkway_max) t = {P.aisle_centre, dep};
        else t = {0.0f, P.pitch_recovery_depth};
        f2 target = alongX ? s * t : s * f2{t.y, t.x};
        f2 toTarget = target - xy(p);
        return length(toTarget) > P.goal_deadzone ? safeNormalize(toTarget, P.safe_eps) : f2{0.0f, 0.0f};
    }

    // cpu_crowd_sim.cpp:662-668
    __device__ __forceinline__ bool exits(float4 p) const {
        float m = smax(fabsf(p.x), fabsf(p.y));
        return (m > V.exhiX && p.z < V.exMaxZ) || m > V.dmaxX;
    }

    // cpu_crowd_sim.cpp:312-332 calcGradient / sceneDist / sceneNormal
    __device__ f3 calcGradient(f3 p) const {
        const f3 kxyy{1.0f, -1.0f, -1.0f}, kyyx{-1.0f, -1.0f, 1.0f}, kyxy{-1.0f, 1.0f, -1.0f}, kxxx{1.0f, 1.0f, 1.0f};
        const float h = P.obstacle_grad_h;
        f3 a = kxyy * map(p + kxyy * h), b = kyyx * map(p + kyyx * h), c = kyxy * map(p + kyxy * h), d = kxxx * map(p + kxxx * h);
        return (a + b + c + d) * P.obstacle_grad_scale;
    }
    __device__ float sceneDist(f3 p, bool& fenceActive) const {
        float dStadium = map(p);
        float dFence = sdFence(p) + P.body_radius;
        fenceActive = dFence < dStadium;
        return fenceActive ? dFence : dStadium;
    }
    __device__ f2 sceneNormal(f3 p, bool fenceActive) const {
        return fenceActive ? sdFenceGradient(p) : xy(safeNormalize(calcGradient(p), P.safe_eps));
    }

    __device__ bool restOnFloor(f3& np, f3& nv, float zFrom) const {   // cpu_crowd_sim.cpp:334-342
        float zFloor;
        if (floorUnderReach(np, zFrom, P.body_radius, zFloor) && np.z < zFloor + P.body_radius) {
            np.z = zFloor + P.body_radius;
            nv.z = 0.0f;
            return true;
        }
        return false;
    }
    __device__ bool settleOnFloor(f3& np, f3& nv, float zFrom) const {   // cpu_crowd_sim.cpp:344-352
        float zFloor;
        if (floorUnderReach(np, zFrom, P.floor_settle_reach, zFloor)) {
            np.z = zFloor + P.body_radius;
            nv.z = 0.0f;
            return true;
        }
        return false;
    }

    // cpu_crowd_sim.cpp:174-184; br = (a, f(a), b, f(b))
    __device__ __forceinline__ static float rootStep(float4& br, float t, float4 g, f3 u) {
        if (g.w > 0.0f) { br.x = t; br.y = g.w; } else { br.z = t; br.w = g.w; }
        float du = dot(f3{g.x, g.y, g.z}, u);
        float tn = du < 0.0f ? t - g.w / du : -1.0f;
        return tn > br.x && tn < br.z ? tn : (br.x * br.w - br.z * br.y) / (br.w - br.y);
    }
    __device__ __forceinline__ static float newtonStep(float t, float4 g, f3 u) {
        float du = dot(f3{g.x, g.y, g.z}, u);
        return du < 0.0f ? t - g.w / du : t;
    }

    // cpu_crowd_sim.cpp:354-382 wallContact
    __device__ float wallContact(f3 np, float fc, f3 u, float fr, float reach, f2& away) const {
        float4 br = make_float4(0.0f, fc, reach, fr);
        float t = reach * fc / (fc - fr);
        float4 g = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (int i = 0; i < P.wall_root_steps; ++i) {
            g = mapExactGrad(np + u * t);
            t = rootStep(br, t, g, u);
        }
        const bool wall = g.z <= P.wall_max_nz * length(f3{g.x, g.y, g.z});
        float e = wall ? t : 1e9f;
        away = f2{-u.x, -u.y};
        f2 n = safeNormalize(f2{g.x, g.y}, P.safe_eps);
        f3 u2{-n.x, -n.y, 0.0f};
        float t2 = 0.0f, t3 = t * dot(u, u2);
        float4 g2 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (int i = 0; i < P.wall_recast_steps; ++i) {
            t2 = t3;
            g2 = mapExactGrad(np + u2 * t2);
            t3 = newtonStep(t2, g2, u2);
        }
        const bool ok = wall && dot(f3{g2.x, g2.y, g2.z}, u2) < 0.0f && fabsf(t3 - t2) < P.wall_recast_tol && t3 > 0.0f &&
                        g2.z <= P.wall_max_nz * length(f3{g2.x, g2.y, g2.z});
        if (ok && t3 < e) { e = t3; away = n; }
        return e;
    }

    // cpu_crowd_sim.cpp:384-441 clearWalls (baked branch)
    __device__ bool clearWalls(f3& np, f3& nv, f3& wall) const {
        bool moved = false;
        wall = f3{0.0f, 0.0f, 0.0f};
        for (int pass = 0; pass < P.wall_passes; ++pass) {
            const bool nearFence = sdFence(np) < P.feeler_reach;
            const float fc = map(np);
            float fr1 = 0.0f, fr2 = 0.0f;
            int i1 = -1, i2 = -1;
            for (int i = 0; i < P.feeler_count; ++i) {
                f3 f = np + f3{P.feeler_off[i][0], P.feeler_off[i][1], 0.0f};
                float v = map(f);
                if (nearFence && sdFence(f) < 0.0f) v = 1.0f;
                if (v < fr1)      { fr2 = fr1; i2 = i1; fr1 = v; i1 = i; }
                else if (v < fr2) { fr2 = v; i2 = i; }
            }
            if (i1 < 0) break;
            f2 hNorm;
            float clearance;
            if (fc > 0.0f) {
                clearance = wallContact(np, fc, f3{P.feeler_dir[i1][0], P.feeler_dir[i1][1], 0.0f}, fr1, P.feeler_reach, hNorm);
                if (i2 >= 0) {
                    f2 h2;
                    float c2 = wallContact(np, fc, f3{P.feeler_dir[i2][0], P.feeler_dir[i2][1], 0.0f}, fr2, P.feeler_reach, h2);
                    if (c2 < clearance) { clearance = c2; hNorm = h2; }
                }
            } else {
                float4 g = mapExactGrad(np);
                hNorm = safeNormalize(f2{g.x, g.y}, P.safe_eps);
                clearance = g.w / smax(length(f2{g.x, g.y}), P.centre_grad_min);
            }
            if (clearance >= P.body_radius) {
                if (clearance < 1e9f) wall = f3{hNorm.x, hNorm.y, clearance - P.body_radius};
                break;
            }
            setXY(np, xy(np) + hNorm * (P.body_radius - clearance));
            moved = true;
            wall = f3{hNorm.x, hNorm.y, 0.0f};
            float vDotN = dot(xy(nv), hNorm);
            if (vDotN < 0.0f) setXY(nv, xy(nv) - hNorm * vDotN);
        }
        return moved;
    }

    // cpu_crowd_sim.cpp:443-461 wallPlaneProbe (baked branch)
    __device__ f3 wallPlaneProbe(f3 np, float) const {
        const bool nearFence = sdFence(np) < P.plane_probe_reach;
        const float fc = map(np);
        float fr = 0.0f;
        int i1 = -1;
        for (int i = 0; i < P.feeler_count; ++i) {
            f3 f = np + f3{P.probe_off[i][0], P.probe_off[i][1], 0.0f};
            float v = map(f);
            if (nearFence && sdFence(f) < 0.0f) v = 1.0f;
            if (v < fr) { fr = v; i1 = i; }
        }
        if (i1 < 0 || fc <= 0.0f) return f3{0.0f, 0.0f, 0.0f};
        f2 away;
        float c = wallContact(np, fc, f3{P.feeler_dir[i1][0], P.feeler_dir[i1][1], 0.0f}, fr, P.plane_probe_reach, away);
        return c < 1e9f ? f3{away.x, away.y, smax(c - P.body_radius, 0.0f)} : f3{0.0f, 0.0f, 0.0f};
    }

    __device__ __forceinline__ bool bakedSolid(f3 p) const { return sdFence(p) >= 0.0f && mapExactGrad(p).w <= 0.0f; }

    // cpu_crowd_sim.cpp:465-479 sweepBack
    __device__ bool sweepBack(f3 pOld, f3& np, f3& nv) const {
        if (!bakedSolid(np)) return false;
        float lo = 0.0f, hi = 1.0f;
        if (!bakedSolid(f3{np.x, np.y, pOld.z})) lo = 1.0f;
        for (int i = 0; i < P.sweep_bisections; ++i) {
            float t = 0.5f * (lo + hi);
            f2 m = mix(xy(pOld), xy(np), t);
            if (bakedSolid(f3{m.x, m.y, pOld.z})) hi = t;
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

    // cpu_crowd_sim.cpp:483-514 resolveStatic
    __device__ bool resolveStatic(f3 pOld, f3& np, f3& nv, bool settle, f3& wall, uint32_t& contact, float) const {
        if (fenceCCD(pOld, np, nv)) contact |= C_FENCE_CCD;
        float dFence = sdFence(np);
        if (dFence < 0.0f) {
            f2 n = sdFenceGradient(np);
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
                f3 w2;
                const bool again = clearWalls(np, nv, w2);
                if (w2.x != 0.0f || w2.y != 0.0f) wall = w2;
                if (again && restOnFloor(np, nv, pOld.z)) contact |= C_FLOOR;
            } else if (restOnFloor(np, nv, pOld.z)) {
                contact |= C_FLOOR;
            }
        }
        return grounded;
    }

    // cpu_crowd_sim.cpp:518-549 stepUpWindow / stepUpBlocked
    __device__ int stepUpWindow(f2 pxy, float f0, float4& g) const {
        const int res = V.sdfRes;
        g = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
        f3 f = toTex(f3{pxy.x, pxy.y, f0});
        const float hiLim = float(res) - 1.0f;
        if (f.x < 0.0f || f.y < 0.0f || f.x > hiLim || f.y > hiLim) return 0;
        const int i0x = smin(int(floorf(f.x)), res - 2), i0y = smin(int(floorf(f.y)), res - 2);
        f2 w{f.x - float(i0x), f.y - float(i0y)};
        const float fLo = f.z + P.step_up_tol * V.sdfInv, fHi = f.z + P.max_step_up * V.sdfInv;
        int k = int(floorf(fHi));
        float a = columnLevel(i0x, i0y, w, k), b = columnLevel(i0x, i0y, w, k + 1);
        if (mix(a, b, fHi - float(k)) <= 0.0f) {
            g = mapExactGrad(f3{pxy.x, pxy.y, V.sdfMinZ + (fHi - 1.0f) / V.sdfInv});
            return 2;
        }
        for (int cell = 0; cell < 2; ++cell) {
            float fBot = smax(float(k), fLo);
            if (mix(a, b, fBot - float(k)) <= 0.0f) {
                float fRoot = float(k) + a / (a - b);
                g = mapExactGrad(f3{pxy.x, pxy.y, V.sdfMinZ + (fRoot - 1.0f) / V.sdfInv});
                return 1;
            }
            if (fBot == fLo) return 0;
            --k; b = a; a = columnLevel(i0x, i0y, w, k);
        }
        return 0;
    }
    __device__ __forceinline__ bool stepUpBlocked(int r, float4 g, f2 dir, bool end) const {
        if (r == 2) return end;
        return r == 1 && dot(f2{g.x, g.y}, dir) < 0.0f && g.z <= P.wall_max_nz * length(f3{g.x, g.y, g.z});
    }
    // cpu_crowd_sim.cpp:555-580 stepUpScan
    __device__ float stepUpScan(f2 p0, f2 p1, float f0, f2& n) const {
        n = f2{0.0f, 0.0f};
        f2 d = p1 - p0;
        float len = length(d);
        f2 dir = len > 0.0f ? d / len : f2{0.0f, 0.0f};
        const int ns = sclamp(int(ceilf(len / P.step_up_sample)), 1, P.step_up_max_samples);
        int lastOk = 0;
        bool blocked = false;
        for (int i = 1; i <= ns; ++i) {
            float4 g;
            int r = stepUpWindow(mix(p0, p1, float(i) / float(ns)), f0, g);
            if (stepUpBlocked(r, g, dir, i == ns)) { blocked = true; n = safeNormalize(f2{g.x, g.y}, P.safe_eps); break; }
            if (r != 2) lastOk = i;
        }
        if (!blocked) return 1.0f;
        float lo = float(lastOk) / float(ns), hi = float(lastOk + 1) / float(ns);
        for (int i = 0; i < P.step_up_bisections; ++i) {
            float t = 0.5f * (lo + hi);
            float4 g;
            int r = stepUpWindow(mix(p0, p1, t), f0, g);
            if (stepUpBlocked(r, g, dir, true)) { hi = t; n = safeNormalize(f2{g.x, g.y}, P.safe_eps); }
            else lo = t;
        }
        return lo;
    }
    // cpu_crowd_sim.cpp:583-613 limitStepUp (baked branch)
    __device__ bool limitStepUp(f3 pOld, f3& np, f3& nv, float) const {
        float f0;
        if (!floorUnderReach(pOld, pOld.z, P.step_up_floor_reach, f0)) f0 = pOld.z - P.step_up_floor_reach;
        f2 n;
        float t = stepUpScan(xy(pOld), xy(np), f0, n);
        if (t >= 1.0f) return false;
        f2 q = mix(xy(pOld), xy(np), t);
        f2 rest = xy(np) - q;
        f2 tangent = rest - n * dot(rest, n);
        float lt = length(tangent);
        if (lt > 0.0f) {
            for (int k = 0; k < P.step_up_slide_tries; ++k) {
                f2 slide = q + tangent * P.step_up_slide[k][0] + n * (lt * P.step_up_slide[k][1]);
                f2 n2;
                if (sdFence(f3{slide.x, slide.y, 0.0f}) >= 0.0f && stepUpScan(q, slide, f0, n2) >= 1.0f) { q = slide; break; }
            }
        }
        float vn = dot(xy(nv), n);
        if (vn < 0.0f) setXY(nv, xy(nv) - n * vn);
        float zFloor;
        if (floorUnderReach(f3{q.x, q.y, pOld.z}, pOld.z, P.floor_settle_reach, zFloor)) {
            np = f3{q.x, q.y, zFloor + P.body_radius};
            nv.z = 0.0f;
        } else {
            np = f3{q.x, q.y, smin(np.z, pOld.z)};
        }
        return true;
    }

    // the projection's fence bound (cpu_crowd_sim.cpp:813-814)
    __device__ __forceinline__ void fenceProject(f3& q) const {
        float dFence = sdFence(q);
        if (dFence < 0.0f) setXY(q, xy(q) - sdFenceGradient(q) * dFence);
    }
    __device__ __forceinline__ float speedFactor(f3) const { return 1.0f; }
};

}  // namespace swarm_gpu
