// The reference's analytic seated venues (S, M, L) on the GPU: a closed-form heightfield of square-ring rows in the
// folded frame (lat = min(|x|, |y|), dep = max(|x|, |y|)), evaluated exactly, with the pitch fence of the terrace, the
// static contacts and step-up limit of the reference's analytic-venue branch, the incline speed and stair spacing, and
// e_goal from the reference's navigation field (its GpuNavCell table). Restated from DedovSergei/swarm-crowd-simulation
// src/venue.cpp (namespace seated, the CPU mirror of shaders/venue_seated.glsl), src/nav_field.cpp and
// src/cpu_crowd_sim.cpp; each function cites its lines there. Float operations follow the CPU code one for one (glm's
// component order, glm::abs as x >= 0 ? x : -x, glm::normalize as v * (1 / sqrt(dot(v, v)))), so the results are the
// reference's bits.
#pragma once

#include "device_math.cuh"
#include "step_args.cuh"
#include "venue_stadium.cuh"

#include <cstring>
#include <vector>

namespace swarm_gpu {

// seated::CellKind (include/swarm/venue.hpp:193)
enum : int { SK_GROUND = 0, SK_TREAD = 1, SK_SEAT = 2, SK_INCLINE = 3, SK_BARRIER = 4, SK_WALL = 5, SK_CONC = 6, SK_SIDE = 7 };
constexpr float SEATED_BIG = 1e9f;
constexpr int SCAN_CROSSINGS = 4, SCAN_BISECTIONS = 12;   // seated::SCAN_CROSSINGS / SCAN_BISECTIONS (venue.hpp:222)

SWARM_HD __forceinline__ float gabs(float x) { return x >= 0.0f ? x : -x; }   // glm::abs on the host (compute_common.hpp)
SWARM_HD __forceinline__ bool operator==(f2 a, f2 b) { return a.x == b.x && a.y == b.y; }   // glm's vec2 ==
SWARM_HD __forceinline__ f2 gnormalize(f2 v) {                                // glm::normalize
    const float r = 1.0f / sqrtf(dot(v, v));
    return {v.x * r, v.y * r};
}
SWARM_HD __forceinline__ f3 gnormalize(f3 v) {
    const float r = 1.0f / sqrtf(dot(v, v));
    return {v.x * r, v.y * r, v.z * r};
}

// The seated venue on the device is one blob: the layout, then its band table ((lo, hi) per band), the first cell of
// each band (bands + 1 entries) and the cell table ((l0, l1, kind, top) per cell), each array 16-byte aligned. The
// tables hold exactly what the band and cell functions compute (SeatedGeom::bandCompute / cellCompute /
// cellTopCompute, the same source compiled for the host), so a lookup gives the computed bits without redoing the
// band walk in every query.
struct SeatedTablesHeader {
    SwarmSeatedLayout layout;
    int32_t bands, cells, band_off, start_off, cell_off, pad[3];   // byte offsets from the blob's start
};

// The constants of the step-up scan (passed by value: the out-of-line functions read no kernel parameter)
struct StepUpConst {
    float sample, tol;
    int maxSamples;
};

// (Out-of-line functions reach the layout through a pointer to global memory: a reference into the kernel's
// parameter space would make every thread copy the parameters to its stack.)
struct SeatedGeom {
    const SwarmSeatedLayout* __restrict__ L;

    SWARM_HD __forceinline__ float rowFront(int k) const { return L->row0 + float(k) * L->row_depth; }   // venue.cpp:417
    SWARM_HD __forceinline__ float rowTread(int k) const { return L->first_row + float(k) * L->row_rise; }
    SWARM_HD __forceinline__ int bandCount() const { return 6 + 2 * L->rows; }   // venue.cpp:486
    SWARM_HD __forceinline__ int activeGangways(int r) const {                  // venue.cpp:329-333
        int n = 0;
        for (int i = 0; i < L->gangways; ++i) n += L->gw_row[i] <= r ? 1 : 0;
        return n;
    }
    SWARM_HD __forceinline__ bool mergedCorner(int r) const {                   // venue.cpp:335-338
        const int n = activeGangways(r);
        return n > 0 && r < L->gw_seated[n - 1];
    }

    // venue.cpp:488-504 (computed; the step reads the venue's band table, built from this)
    SWARM_HD void bandCompute(int j, float& lo, float& hi) const {
        const int nb = bandCount();
        if (j <= 0) { lo = 0.0f; hi = L->stand_front; return; }
        if (j == 1) { lo = L->stand_front; hi = L->row0; return; }
        if (j < nb - 4) {
            const int k = (j - 2) >> 1;
            const float d = rowFront(k);
            if (((j - 2) & 1) == 0) { lo = d; hi = d + L->clearway; }
            else { lo = d + L->clearway; hi = rowFront(k + 1); }
            return;
        }
        if (j == nb - 4) { lo = L->conc_front; hi = L->conc_back; return; }
        if (j == nb - 3) { lo = L->conc_back; hi = L->outer_face; return; }
        if (j == nb - 2) { lo = L->outer_face; hi = L->landing_end; return; }
        lo = L->landing_end;
        hi = SEATED_BIG;
    }

    // venue.cpp:506-520
    SWARM_HD int bandOf(float dep) const {
        const int nb = bandCount();
        if (dep < L->stand_front) return 0;
        if (dep < L->row0) return 1;
        if (dep < L->conc_front) {
            int k = sclamp(int(floorf((dep - L->row0) / L->row_depth)), 0, L->rows - 1);
            if (dep < rowFront(k)) --k;
            else if (k + 1 < L->rows && dep >= rowFront(k + 1)) ++k;
            return 2 + 2 * k + (dep >= rowFront(k) + L->clearway ? 1 : 0);
        }
        if (dep < L->conc_back) return nb - 4;
        if (dep < L->outer_face) return nb - 3;
        if (dep < L->landing_end) return nb - 2;
        return nb - 1;
    }

    // venue.cpp:522-594: cell c of band j, ascending in lat (computed; the step reads the venue's cell table)
    SWARM_HD bool cellCompute(int j, int c, float& l0, float& l1, int& kind, int& row) const {
        const int nb = bandCount();
        float lo, hi;
        bandCompute(j, lo, hi);
        row = -1;
        if (j == 0 || j == nb - 1) {
            if (c > 0) return false;
            l0 = 0.0f; l1 = hi; kind = SK_GROUND;
            return true;
        }
        const bool cornerDoor = L->corner_door_lo < 1e8f;
        if (j == nb - 2) {
            const int i = c >> 1;
            if (i < L->doors) {
                if ((c & 1) == 0) { l0 = i == 0 ? 0.0f : L->door_hi[i - 1]; l1 = L->door_lo[i]; kind = SK_GROUND; }
                else { l0 = L->door_lo[i]; l1 = L->door_hi[i]; kind = SK_CONC; }
                return true;
            }
            if (c == 2 * L->doors) { l0 = L->door_hi[L->doors - 1]; l1 = cornerDoor ? L->corner_door_lo : hi; kind = SK_GROUND; return true; }
            if (c == 2 * L->doors + 1 && cornerDoor) { l0 = L->corner_door_lo; l1 = hi; kind = SK_CONC; return true; }
            return false;
        }
        if (c == 0) { l0 = 0.0f; l1 = L->avenue_half; kind = SK_GROUND; return true; }
        if (j == nb - 3) {
            const int i = (c - 1) >> 1;
            if (i < L->doors) {
                if ((c & 1) == 1) { l0 = i == 0 ? L->avenue_half : L->door_hi[i - 1]; l1 = L->door_lo[i]; kind = SK_WALL; }
                else { l0 = L->door_lo[i]; l1 = L->door_hi[i]; kind = SK_CONC; }
                return true;
            }
            if (c == 2 * L->doors + 1) { l0 = L->door_hi[L->doors - 1]; l1 = cornerDoor ? L->corner_door_lo : hi; kind = SK_WALL; return true; }
            if (c == 2 * L->doors + 2 && cornerDoor) { l0 = L->corner_door_lo; l1 = hi; kind = SK_CONC; return true; }
            return false;
        }
        if (j == nb - 4) {
            if (c == 1) { l0 = L->avenue_half; l1 = L->lat0; kind = SK_WALL; return true; }
            if (c > 2) return false;
            l0 = L->lat0; l1 = hi; kind = SK_CONC;
            return true;
        }
        int segKind = SK_BARRIER, gapKind = SK_GROUND;
        bool seatBand = true;
        float corner = hi - L->corner_inset - L->seat_inset;
        if (j >= 2) {
            row = (j - 2) >> 1;
            seatBand = ((j - 2) & 1) != 0;
            segKind = seatBand ? SK_SEAT : SK_TREAD;
            gapKind = SK_INCLINE;
            if (!seatBand) corner = lo - L->corner_inset;
        }
        if (c == 1) { l0 = L->avenue_half; l1 = L->lat0; kind = SK_SIDE; return true; }
        const int r = (j - 1) >> 1;
        const int n = activeGangways(r);
        const bool merged = mergedCorner(r);
        const int i = (c - 2) >> 1;
        if (i < n) {
            if ((c & 1) == 0) {
                l0 = i == 0 ? L->lat0 : (seatBand ? L->gw_hi[i - 1] + L->seat_inset : L->gw_hi[i - 1]);
                l1 = seatBand ? L->gw_lo[i] - L->seat_inset : L->gw_lo[i];
                kind = segKind;
            } else {
                l0 = seatBand ? L->gw_lo[i] - L->seat_inset : L->gw_lo[i];
                l1 = merged && i == n - 1 ? hi : (seatBand ? L->gw_hi[i] + L->seat_inset : L->gw_hi[i]);
                kind = gapKind;
            }
            return true;
        }
        if (merged) return false;
        if (c == 2 + 2 * n) { l0 = seatBand ? L->gw_hi[n - 1] + L->seat_inset : L->gw_hi[n - 1]; l1 = corner; kind = segKind; return true; }
        if (c == 3 + 2 * n) { l0 = corner; l1 = hi; kind = gapKind; return true; }
        return false;
    }

    // venue.cpp:596-607 (computed; the cell table holds each cell's top, an incline's excepted)
    SWARM_HD float cellTopCompute(int kind, int row, float dep) const {
        switch (kind) {
        case SK_TREAD: return rowTread(row);
        case SK_SEAT: return rowTread(row) + L->seat_top;
        case SK_INCLINE: return L->rake * (dep - L->row0);
        case SK_BARRIER: return L->barrier_top;
        case SK_WALL: return L->wall_top;
        case SK_CONC: return L->concourse_z;
        case SK_SIDE: return row < 0 ? L->barrier_top : rowTread(row) + L->seat_top;
        default: return 0.0f;
        }
    }

    // ---- the band and cell tables (the step's lookups) ----
    SWARM_HD __forceinline__ const SeatedTablesHeader& H() const { return *reinterpret_cast<const SeatedTablesHeader*>(L); }
    SWARM_HD __forceinline__ const char* base() const { return reinterpret_cast<const char*>(L); }
    SWARM_HD __forceinline__ void band(int j, float& lo, float& hi) const {
        const float2 b = reinterpret_cast<const float2*>(base() + H().band_off)[j];
        lo = b.x;
        hi = b.y;
    }
    // cell c of band j: its lateral bounds, kind and top height (cellTopCompute at dep 0: exact but for an incline)
    SWARM_HD __forceinline__ bool cell(int j, int c, float& l0, float& l1, int& kind, float& top) const {
        const int32_t* start = reinterpret_cast<const int32_t*>(base() + H().start_off);
        const int e = start[j] + c;
        if (e >= start[j + 1]) return false;
        const float4 t = reinterpret_cast<const float4*>(base() + H().cell_off)[e];
        l0 = t.x;
        l1 = t.y;
        int32_t k;
        memcpy(&k, &t.z, 4);
        kind = k;
        top = t.w;
        return true;
    }
    SWARM_HD __forceinline__ float cellTop(int kind, float top, float dep) const {
        return kind == SK_INCLINE ? L->rake * (dep - L->row0) : top;
    }

    // venue.cpp:421-430: the cell of band j containing lat
    SWARM_HD int ownCell(int j, float lat, float& l0, float& l1, int& kind, float& row) const {
        int c = 0;
        float a, b;
        int k;
        float r;
        for (; cell(j, c, a, b, k, r); ++c) {
            l0 = a; l1 = b; kind = k; row = r;
            if (lat < b) return c;
        }
        return c - 1;
    }

    SWARM_HD __forceinline__ static f2 fold(f2 p) {   // venue.cpp:609-612
        const f2 a{gabs(p.x), gabs(p.y)};
        return {smin(a.x, a.y), smax(a.x, a.y)};
    }
    SWARM_HD __forceinline__ static f2 unfoldDir(f2 p, f2 d) {   // venue.cpp:614-618
        const f2 s{p.x < 0.0f ? -1.0f : 1.0f, p.y < 0.0f ? -1.0f : 1.0f};
        const f2 a{gabs(p.x), gabs(p.y)};
        return a.y >= a.x ? f2{s.x * d.x, s.y * d.y} : f2{s.x * d.y, s.y * d.x};
    }

    // venue.cpp:631-638 cellKey, 672-679 floorHeight
    SWARM_HD __noinline__ f2 cellKey(f2 p) const {
        const f2 f = fold(p);
        const int j = bandOf(f.y);
        float l0, l1;
        int kind;
        float row;
        ownCell(j, f.x, l0, l1, kind, row);
        return {float(j), l0};
    }
    SWARM_HD __noinline__ float floorHeight(f2 p) const {
        const f2 f = fold(p);
        const int j = bandOf(f.y);
        float l0, l1;
        int kind;
        float row;
        ownCell(j, f.x, l0, l1, kind, row);
        return cellTop(kind, row, f.y);
    }

    // venue.cpp:640-650 floorSlope: the floor's rise per unit of travel along e (0 off the inclines)
    SWARM_HD __noinline__ float floorSlope(f2 p, f2 e) const {
        const f2 f = fold(p);
        const int j = bandOf(f.y);
        float l0, l1;
        int kind;
        float row;
        ownCell(j, f.x, l0, l1, kind, row);
        if (kind != SK_INCLINE) return 0.0f;
        const f2 g = unfoldDir(p, f2{0.0f, L->rake});
        const float a = g.x * e.x, b = g.y * e.y;
        return a + b;
    }

    // venue.cpp:434-449 nearestRegion2
    SWARM_HD static f2 nearestRegion2(float u, float z, float u0, float u1, float s, float uRef, bool below) {
        const float uc = sclamp(u, u0, u1);
        const float tc = s * (uc - uRef);
        if (below ? z <= tc : z >= tc) return {uc, z};
        const float t0 = s * (u0 - uRef), t1 = s * (u1 - uRef);
        const float du = u1 - u0, dz = t1 - t0;
        const float len2 = du * du + dz * dz;
        const float t = len2 > 0.0f ? sclamp(((u - u0) * du + (z - t0) * dz) / len2, 0.0f, 1.0f) : 0.0f;
        f2 best{u0 + t * du, t0 + t * dz};
        float bd = (u - best.x) * (u - best.x) + (z - best.y) * (z - best.y);
        const f2 r0{u0, below ? smin(z, t0) : smax(z, t0)}, r1{u1, below ? smin(z, t1) : smax(z, t1)};
        const float d0 = (u - r0.x) * (u - r0.x) + (z - r0.y) * (z - r0.y), d1 = (u - r1.x) * (u - r1.x) + (z - r1.y) * (z - r1.y);
        if (d0 < bd) { bd = d0; best = r0; }
        if (d1 < bd) { best = r1; }
        return best;
    }

    // venue.cpp:456-477 nearestInCell: the nearest point of a cell's solid (or air) column; squared distance in .w
    SWARM_HD float4 nearestInCell(float lo, float hi, float l0, float l1, int kind, float row, f3 pf, bool airColumn) const {
        const float latC = sclamp(pf.x, l0, l1);
        f3 q;
        if (kind == SK_INCLINE) {
            const f2 n2 = nearestRegion2(pf.y, pf.z, lo, hi, L->rake, L->row0, !airColumn);
            q = f3{latC, n2.x, n2.y};
            if (airColumn && q.x > q.y) {
                const float s0 = smax(l0, lo), s1 = smin(l1, hi);
                if (s0 > s1) return make_float4(q.x, q.y, q.z, SEATED_BIG);
                const float r2 = 1.41421356f;
                const float m = 0.5f * (pf.x + pf.y);
                const f2 w = nearestRegion2(m * r2, pf.z, s0 * r2, s1 * r2, L->rake / r2, L->row0 * r2, false);
                const float s = w.x / r2;
                q = f3{s, s, w.y};
            }
        } else {
            const float top = cellTop(kind, row, 0.0f);
            q = f3{latC, sclamp(pf.y, lo, hi), airColumn ? smax(pf.z, top) : smin(pf.z, top)};
        }
        const f3 d = pf - q;
        return make_float4(q.x, q.y, q.z, dot(d, d));
    }

    // venue.cpp:690-751 sdfGradStats: exact signed distance to the heightfield and its gradient (gradient, value)
    SWARM_HD __noinline__ float4 sdfGrad(f3 p) const {
        const f2 f = fold(xy(p));
        const f3 pf{f.x, f.y, p.z};
        const int nb = bandCount();
        const int jp = bandOf(pf.y);
        float l0, l1;
        int kind;
        float row;
        ownCell(jp, pf.x, l0, l1, kind, row);
        const bool inAir = pf.z > cellTop(kind, row, pf.y);
        float best = SEATED_BIG;
        f3 bestQ = pf;
        float4 bestRect = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        int bestKind = kind;
        auto visit = [&](int j, float g2) {
            float lo, hi;
            band(j, lo, hi);
            float a, b;
            int k;
            float r;
            for (int c = 0; cell(j, c, a, b, k, r); ++c) {
                const float lg = smax(smax(a - pf.x, pf.x - b), 0.0f);
                if (g2 + lg * lg >= best) {
                    if (a > pf.x) break;
                    continue;
                }
                const float4 n = nearestInCell(lo, hi, a, b, k, r, pf, !inAir);
                if (n.w < best) { best = n.w; bestQ = f3{n.x, n.y, n.z}; bestRect = make_float4(a, b, lo, hi); bestKind = k; }
            }
        };
        visit(jp, 0.0f);
        bool down = true, up = true;
        for (int s = 1; s <= L->max_band_steps && (down || up); ++s) {
            for (int side = 0; side < 2; ++side) {
                bool& open = side == 0 ? down : up;
                if (!open) continue;
                const int j = side == 0 ? jp - s : jp + s;
                if (j < 0 || j >= nb) { open = false; continue; }
                float lo, hi;
                band(j, lo, hi);
                const float g = smax(smax(lo - pf.y, pf.y - hi), 0.0f);
                if (g * g >= best) { open = false; continue; }
                visit(j, g * g);
            }
        }
        const float d = sqrtf(best);
        f3 gf;
        if (d > 0.0f) {
            const f3 t = inAir ? pf - bestQ : bestQ - pf;
            gf = f3{t.x / d, t.y / d, t.z / d};
        } else {
            const float sgn = inAir ? -1.0f : 1.0f;
            const f2 h{pf.x <= bestRect.x ? sgn : pf.x >= bestRect.y ? -sgn : 0.0f,
                       pf.y <= bestRect.z ? sgn : pf.y >= bestRect.w ? -sgn : 0.0f};
            if (h.x != 0.0f || h.y != 0.0f) {
                const f2 hn = gnormalize(h);
                gf = f3{hn.x, hn.y, 0.0f};
            } else {
                gf = bestKind == SK_INCLINE ? gnormalize(f3{0.0f, -L->rake, 1.0f}) : f3{0.0f, 0.0f, 1.0f};
            }
        }
        const f2 g = unfoldDir(xy(p), f2{gf.x, gf.y});
        return make_float4(g.x, g.y, gf.z, inAir ? d : -d);
    }

    // venue.cpp:753-804 wall: the nearest wall in the plane z = c.z (direction away from it, clearance), or WALL_NONE
    SWARM_HD __noinline__ f3 wall(f3 c, float reach) const {
        const f2 f = fold(xy(c));
        const int nb = bandCount();
        const int jp = bandOf(f.y);
        float l0, l1;
        int kind;
        float row;
        ownCell(jp, f.x, l0, l1, kind, row);
        const bool inWall = kind != SK_INCLINE && cellTop(kind, row, f.y) > c.z;
        float best = inWall ? SEATED_BIG : reach * reach;
        f2 bestQ = f;
        float4 bestRect = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        bool found = false;
        auto visit = [&](int j) {
            float lo, hi;
            band(j, lo, hi);
            float a, b;
            int k;
            float r;
            for (int cc = 0; cell(j, cc, a, b, k, r); ++cc) {
                const bool isWall = k != SK_INCLINE && cellTop(k, r, lo) > c.z;
                if (isWall == inWall) continue;
                const f2 q{sclamp(f.x, a, b), sclamp(f.y, lo, hi)};
                const f2 dd = f - q;
                const float d2 = dot(dd, dd);
                if (d2 < best) { best = d2; bestQ = q; bestRect = make_float4(a, b, lo, hi); found = true; }
            }
        };
        visit(jp);
        bool down = true, up = true;
        for (int s = 1; s <= L->max_band_steps && (down || up); ++s) {
            for (int side = 0; side < 2; ++side) {
                bool& open = side == 0 ? down : up;
                if (!open) continue;
                const int j = side == 0 ? jp - s : jp + s;
                if (j < 0 || j >= nb) { open = false; continue; }
                float lo, hi;
                band(j, lo, hi);
                const float g = smax(smax(lo - f.y, f.y - hi), 0.0f);
                if (g * g >= best) { open = false; continue; }
                visit(j);
            }
        }
        if (!found) return f3{0.0f, 0.0f, WALL_NONE};
        const float d = sqrtf(best);
        f2 dir;
        if (d > 0.0f) {
            const f2 t = inWall ? bestQ - f : f - bestQ;
            dir = t / d;
        } else {
            const float sgn = inWall ? 1.0f : -1.0f;
            dir = gnormalize(f2{f.x <= bestRect.x ? sgn : f.x >= bestRect.y ? -sgn : 0.0f,
                                f.y <= bestRect.z ? sgn : f.y >= bestRect.w ? -sgn : 0.0f});
        }
        const f2 u = unfoldDir(xy(c), dir);
        return f3{u.x, u.y, inWall ? -d : d};
    }

    // venue.cpp:807-835 stepUpScan: the fraction of the move p0 -> p1 an agent whose start floor is f0 may take
    SWARM_HD __noinline__ float stepUpScan(StepUpConst P, f2 p0, f2 p1, float f0, f2& n) const {
        n = f2{0.0f, 0.0f};
        const float len = length(p1 - p0);
        const int ns = sclamp(int(ceilf(len / P.sample)), 1, P.maxSamples);
        float lo = 0.0f;
        f2 key = cellKey(p0);
        for (int i = 1; i <= ns; ++i) {
            const float t = float(i) / float(ns);
            for (int k = 0; k < SCAN_CROSSINGS; ++k) {
                if (cellKey(mix(p0, p1, t)) == key) break;
                float a = lo, b = t;
                for (int m = 0; m < SCAN_BISECTIONS; ++m) {
                    const float tm = 0.5f * (a + b);
                    if (cellKey(mix(p0, p1, tm)) == key) a = tm;
                    else b = tm;
                }
                const float ha = floorHeight(mix(p0, p1, a)), hb = floorHeight(mix(p0, p1, b));
                if (hb > f0 + P.tol && hb - ha > L->rake * len * (b - a) + P.tol) {
                    const f2 pa = mix(p0, p1, a);
                    const f3 w = wall(f3{pa.x, pa.y, ha + P.tol}, P.sample);
                    n = w.z < WALL_NONE ? f2{w.x, w.y} : (p0 - p1) / smax(len, 1e-30f);
                    return a;
                }
                lo = b;
                key = cellKey(mix(p0, p1, b));
            }
            lo = t;
        }
        return 1.0f;
    }

    // cpu_crowd_sim.cpp:264-270: the heightfield's floor under c (the step's floorUnderReach on a seated venue)
    SWARM_HD __forceinline__ bool floorUnderReach(f3 c, float zFrom, float down, float bodyRadius, float& zFloor) const {
        const float h = floorHeight(xy(c));
        zFloor = h;
        if (c.z <= h) return h <= smax(zFrom, c.z) + bodyRadius;
        return h >= c.z - down;
    }

    // cpu_crowd_sim.cpp:601-617 venueBlockedWall: a blocked move's point may lie in a wall's clearance band; the wall
    // contact there, kept only if the push climbs no face
    SWARM_HD __noinline__ void blockedWall(StepUpConst su, float feelerReach, float bodyRadius, float settleReach, float f0,
                                           f3 pOld, f3& np, f3& nv) const {
        const f3 w = wall(np + f3{0.0f, 0.0f, L->wall_above}, feelerReach);
        if (w.z >= L->wall_clear) return;
        const f2 pushed = xy(np) + f2{w.x, w.y} * (L->wall_clear - w.z);
        f2 n;
        if (stepUpScan(su, xy(np), pushed, f0, n) < 1.0f) return;
        const float vDotN = dot(xy(nv), f2{w.x, w.y});
        if (vDotN < 0.0f) setXY(nv, xy(nv) - f2{w.x, w.y} * vDotN);
        float zFloor;
        if (floorUnderReach(f3{pushed.x, pushed.y, pOld.z}, pOld.z, settleReach, bodyRadius, zFloor)) {
            np = f3{pushed.x, pushed.y, zFloor + bodyRadius};
            nv.z = 0.0f;
        } else {
            setXY(np, pushed);
        }
    }

    // cpu_crowd_sim.cpp:622-650 venueEdgeMargin: every centre face_margin off the side face of a column higher than its
    // feet; on such a column's edge: onto it unless that climbs; lifted and left over a lower floor: settled from the
    // start-of-step height; airborne: off the face, still falling
    SWARM_HD __noinline__ void edgeMargin(StepUpConst su, float bodyRadius, float settleReach, f3 pOld, float f0, f3& np,
                                          f3& nv) const {
        const float margin = L->face_margin;
        float feet = np.z - bodyRadius;
        const float fl = floorHeight(xy(np));
        if (feet > fl + margin) {
            const f3 w = wall(f3{np.x, np.y, fl + su.tol}, margin);
            if (w.z < margin) {
                const f2 into = xy(np) - f2{w.x, w.y} * (w.z + margin);
                const float top = floorHeight(into);
                if (fabsf(top - feet) <= margin && top <= f0 + su.tol) { setXY(np, into); return; }
            }
            if (np.z <= pOld.z) {
                const f3 wa = wall(f3{np.x, np.y, feet + su.tol}, margin);
                if (wa.z < margin) setXY(np, xy(np) + f2{wa.x, wa.y} * (margin - wa.z));
                return;
            }
            float zFloor;
            if (!floorUnderReach(f3{np.x, np.y, pOld.z}, pOld.z, settleReach, bodyRadius, zFloor)) { np.z = pOld.z; return; }
            np.z = zFloor + bodyRadius;
            nv.z = 0.0f;
            feet = zFloor;
        }
        const f3 w = wall(f3{np.x, np.y, feet + su.tol}, margin);
        if (w.z >= margin) return;
        setXY(np, xy(np) + f2{w.x, w.y} * (margin - w.z));
        np.z = floorHeight(xy(np)) + bodyRadius;
    }
};


// The seated venue's device blob for a layout (a host function): the layout, its band table and its cell table
inline std::vector<unsigned char> seatedBlob(const SwarmSeatedLayout& layout) {
    SeatedTablesHeader h{};
    h.layout = layout;
    const SeatedGeom G{&h.layout};
    const int nb = G.bandCount();
    std::vector<float2> bands(static_cast<size_t>(nb));
    std::vector<int32_t> start(static_cast<size_t>(nb) + 1, 0);
    std::vector<float4> cells;
    for (int j = 0; j < nb; ++j) {
        G.bandCompute(j, bands[size_t(j)].x, bands[size_t(j)].y);
        start[size_t(j)] = int32_t(cells.size());
        float l0, l1;
        int kind, row;
        for (int c = 0; G.cellCompute(j, c, l0, l1, kind, row); ++c) {
            float4 t;
            t.x = l0;
            t.y = l1;
            const int32_t kk = kind;
            memcpy(&t.z, &kk, 4);
            t.w = kind == SK_INCLINE ? 0.0f : G.cellTopCompute(kind, row, 0.0f);
            cells.push_back(t);
        }
    }
    start[size_t(nb)] = int32_t(cells.size());
    auto up16 = [](size_t x) { return (x + 15) / 16 * 16; };
    h.bands = nb;
    h.cells = int32_t(cells.size());
    h.band_off = int32_t(up16(sizeof h));
    h.start_off = int32_t(up16(size_t(h.band_off) + bands.size() * sizeof(float2)));
    h.cell_off = int32_t(up16(size_t(h.start_off) + start.size() * sizeof(int32_t)));
    std::vector<unsigned char> blob(size_t(h.cell_off) + cells.size() * sizeof(float4), 0);
    memcpy(blob.data(), &h, sizeof h);
    memcpy(blob.data() + h.band_off, bands.data(), bands.size() * sizeof(float2));
    memcpy(blob.data() + h.start_off, start.data(), start.size() * sizeof(int32_t));
    memcpy(blob.data() + h.cell_off, cells.data(), cells.size() * sizeof(float4));
    return blob;
}

// The navigation field's lookup (src/nav_field.cpp:375-441; physics.comp navCell / navDirection / navGoal): cells of
// the reference's GpuNavCell (anchor x, anchor y, distance, info bits), res x res, x fastest
SWARM_HD __forceinline__ float4 loadCell(const float4* p) {
#ifdef __CUDA_ARCH__
    return __ldg(p);
#else
    return *p;
#endif
}

struct SeatedNav {
    SeatedGeom G;
    StepUpConst su;
    float goalDeadzone, feelerReach, safeEps;
    const float4* cells;
    int res;
    float origin, cell, inv;

    SWARM_HD __forceinline__ uint32_t info(int i) const {
        const float w = loadCell(cells + i).w;
        uint32_t u;
        memcpy(&u, &w, 4);
        return u;
    }
    SWARM_HD __forceinline__ f2 cellCentre(int i) const {   // nav_field.cpp:375-379 surfaceCellCentre
        const float cx = float(i % res) + 0.5f, cy = float(i / res) + 0.5f;
        const float px = cx * cell, py = cy * cell;
        return {origin + px, origin + py};
    }
    SWARM_HD __forceinline__ bool reaches(f2 x, f2 c) const {   // nav_field.cpp:381-385 surfaceReaches
        if (G.cellKey(c) == G.cellKey(x)) return true;
        f2 n;
        return G.stepUpScan(su, x, c, G.floorHeight(x), n) >= 1.0f;
    }
    // nav_field.cpp:387-421 directionCell: the cell containing x, or its nearest FIT neighbour with a path when it is
    // NOFIT; then the surface rule (the nearest such cell whose centre the agent may walk straight to)
    SWARM_HD __noinline__ int cellOf(f2 x) const {
        const f2 g{(x.x - origin) * inv, (x.y - origin) * inv};
        const int cx = sclamp(int(floorf(g.x)), 0, res - 1), cy = sclamp(int(floorf(g.y)), 0, res - 1);
        int i = cx + cy * res;
        constexpr uint32_t FR = SWARM_NAV_FIT | SWARM_NAV_REACHABLE;
        if ((info(i) & SWARM_NAV_FIT) == 0u) {
            float best = 1e9f;
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    const int mx = cx + dx, my = cy + dy;
                    if ((dx == 0 && dy == 0) || mx < 0 || my < 0 || mx >= res || my >= res) continue;
                    const int j = mx + my * res;
                    if ((info(j) & FR) != FR) continue;
                    const f2 q{g.x - (float(mx) + 0.5f), g.y - (float(my) + 0.5f)};
                    const float d2 = q.x * q.x + q.y * q.y;
                    if (d2 < best) { best = d2; i = j; }
                }
        }
        if (!reaches(x, cellCentre(i))) {
            float best = 1e9f;
            int pick = i;
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    const int mx = cx + dx, my = cy + dy;
                    if (mx < 0 || my < 0 || mx >= res || my >= res) continue;
                    const int j = mx + my * res;
                    if (j == i || (info(j) & FR) != FR) continue;
                    const f2 q{g.x - (float(mx) + 0.5f), g.y - (float(my) + 0.5f)};
                    const float d2 = q.x * q.x + q.y * q.y;
                    if (d2 < best && reaches(x, cellCentre(j))) { best = d2; pick = j; }
                }
            i = pick;
        }
        return i;
    }
    // nav_field.cpp:423-441 direction / goal: the unit vector to the cell's anchor, its component into a wall or step
    // face beside the agent removed
    SWARM_HD __noinline__ f2 goal(f3 p) const {
        const f2 x = xy(p);
        const float4 c = loadCell(cells + cellOf(x));
        f2 e{0.0f, 0.0f};
        uint32_t ci;
        memcpy(&ci, &c.w, 4);
        if (ci & SWARM_NAV_REACHABLE) {
            const f2 d = f2{c.x, c.y} - x;
            const float l = length(d);
            e = l > goalDeadzone ? d / l : f2{0.0f, 0.0f};
        }
        const f3 w = G.wall(p, feelerReach);
        const float into = dot(e, f2{w.x, w.y});
        if (w.z < feelerReach && into < 0.0f) {
            e = e - f2{w.x, w.y} * into;
            const float l = length(e);
            e = l > safeEps ? e / l : f2{0.0f, 0.0f};
        }
        return e;
    }
};

// The queue-aware exit choice's table lookup (src/exit_choice.cpp:512-578; physics.comp navChoiceCell /
// navChoiceDirection / navChoiceGoal): the reference's ChoiceTable on the navigation grid -- per cell an index word
// (SWARM_CHOICE_INDEX_FIT | its entry + 1) and per entry the GpuNavChoiceCell's 36 words (24 slots: anchor bits 0-24,
// exit bits 25-30; then 12 words of two 16-bit distances)
SWARM_HD __forceinline__ uint32_t loadWord(const uint32_t* p) {
#ifdef __CUDA_ARCH__
    return __ldg(p);
#else
    return *p;
#endif
}

constexpr uint32_t CHOICE_SLOT_EMPTY = 63u;   // the exit id of an empty slot (nav::CHOICE_EMPTY)

struct SeatedChoice {
    SeatedNav nav;                 // the grid, the surface rule and the goal's constants (its cells are not read)
    const uint32_t* index;
    const uint32_t* entries;

    SWARM_HD __forceinline__ bool fit(int i) const { return (loadWord(index + i) & SWARM_CHOICE_INDEX_FIT) != 0u; }
    SWARM_HD __forceinline__ bool reachable(int i) const { return (loadWord(index + i) & SWARM_CHOICE_INDEX_MASK) != 0u; }
    // cell i's candidates (36 words), or null for a cell without any (ChoiceTable::at's empty cell)
    SWARM_HD __forceinline__ const uint32_t* entry(int i) const {
        const uint32_t e = loadWord(index + i) & SWARM_CHOICE_INDEX_MASK;
        return e ? entries + size_t(e - 1u) * 36u : nullptr;
    }
    // choiceCell (:512-548): the cell containing x; a NOFIT cell takes the FIT cell with candidates of its 3 x 3 ring
    // whose centre is nearest, else of the 5 x 5 ring's outer cells; then the surface rule over the 3 x 3 cells
    SWARM_HD __forceinline__ bool fitPath(int j) const { return fit(j) && reachable(j); }
    SWARM_HD __noinline__ int cellOf(f2 x) const {
        const int res = nav.res;
        const f2 g{(x.x - nav.origin) * nav.inv, (x.y - nav.origin) * nav.inv};
        const int cx = sclamp(int(floorf(g.x)), 0, res - 1), cy = sclamp(int(floorf(g.y)), 0, res - 1);
        const int i = ringPick(g, cx, cy);
        return surfacePick(x, g, cx, cy, i);
    }
    SWARM_HD __forceinline__ int ringPick(f2 g, int cx, int cy) const {
        const int res = nav.res;
        int i = cx + cy * res;
        if (!fit(i)) {
            float best = 1e9f;
            for (int r = 1; r <= 2 && best == 1e9f; r++)
                for (int dy = -r; dy <= r; dy++)
                    for (int dx = -r; dx <= r; dx++) {
                        if (max(abs(dx), abs(dy)) != r) continue;
                        const int mx = cx + dx, my = cy + dy;
                        if (mx < 0 || my < 0 || mx >= res || my >= res) continue;
                        const int j = mx + my * res;
                        if (!fit(j) || !reachable(j)) continue;
                        const f2 q{g.x - (float(mx) + 0.5f), g.y - (float(my) + 0.5f)};
                        const float d2 = q.x * q.x + q.y * q.y;
                        if (d2 < best) { best = d2; i = j; }
                    }
        }
        return i;
    }
    SWARM_HD __forceinline__ int surfacePick(f2 x, f2 g, int cx, int cy, int i) const {
        const int res = nav.res;
        if (nav.reaches(x, nav.cellCentre(i))) return i;
        float best = 1e9f;
        int pick = i;
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                const int mx = cx + dx, my = cy + dy;
                if (mx < 0 || my < 0 || mx >= res || my >= res) continue;
                const int j = mx + my * res;
                if (j == i || !fitPath(j)) continue;
                const f2 q{g.x - (float(mx) + 0.5f), g.y - (float(my) + 0.5f)};
                const float d2 = q.x * q.x + q.y * q.y;
                if (d2 < best && nav.reaches(x, nav.cellCentre(j))) { best = d2; pick = j; }
            }
        return pick;
    }
    // choiceDirection / choiceGoal (:557-578): towards the anchor of the exit's own field in x's choice cell (its centre
    // in float, anchorCentre :550-555), 0 within the dead zone or when the exit is no candidate there; the component
    // into a wall or step face beside the agent removed
    SWARM_HD __noinline__ f2 goal(f3 p, uint32_t exit) const { return goalFromCell(p, exit, cellOf(xy(p))); }
    // the same for an agent whose choice cell is known (the choice pass's, for the same position)
    SWARM_HD __noinline__ f2 goalFromCell(f3 p, uint32_t exit, int cell_) const {
        const f2 x = xy(p);
        const uint32_t* c = entry(cell_);
        f2 e{0.0f, 0.0f};
        if (c) {
            for (int k = 0; k < 24; ++k) {
                const uint32_t w = loadWord(c + k);
                if (((w >> 25) & 63u) != exit) continue;   // (an exit appears at most once)
                const uint32_t a = w & ((1u << 25) - 1u);
                const float ax = float(a % uint32_t(nav.res)) + 0.5f, ay = float(a / uint32_t(nav.res)) + 0.5f;
                const float px = ax * nav.cell, py = ay * nav.cell;
                const f2 d = f2{nav.origin + px, nav.origin + py} - x;
                const float l = length(d);
                e = l > nav.goalDeadzone ? d / l : f2{0.0f, 0.0f};
                break;
            }
        }
        const f3 w = nav.G.wall(p, nav.feelerReach);
        const float into = dot(e, f2{w.x, w.y});
        if (w.z < nav.feelerReach && into < 0.0f) {
            e = e - f2{w.x, w.y} * into;
            const float l = length(e);
            e = l > nav.safeEps ? e / l : f2{0.0f, 0.0f};
        }
        return e;
    }
};

#ifdef __CUDACC__
// choiceCell by a lane group (G lanes, sub the lane's index in it, the group's lanes adjacent; the whole warp calls it
// together): the ring's pick and its surface check by the group's first lane; only when the agent may not walk straight
// to the pick's centre, the rule's other reach checks -- each of the 3 x 3 cells (t = 3 (dy + 1) + dx + 1) it may visit
// -- shared out over the lanes (check t by lane t mod G), their bits combined over the group, and the rule's choice
// made from them in its own order: the cell cellOf gives. act: the lane's agent takes part (the others only join the
// shuffles).
__device__ __forceinline__ int choiceCellLanes(const SeatedChoice& sc, f2 x, bool act, int G, int sub) {
    const SeatedNav& nav = sc.nav;
    const int res = nav.res;
    const int base = int(threadIdx.x & 31u) - sub;
    const f2 g{(x.x - nav.origin) * nav.inv, (x.y - nav.origin) * nav.inv};
    const int cx = sclamp(int(floorf(g.x)), 0, res - 1), cy = sclamp(int(floorf(g.y)), 0, res - 1);
    const int i = act ? sc.ringPick(g, cx, cy) : cx + cy * res;
    int direct = 1;
    if (act && sub == 0) direct = nav.reaches(x, nav.cellCentre(i)) ? 1 : 0;
    direct = __shfl_sync(0xffffffffu, direct, base);
    const bool search = act && !direct;
    uint32_t bits = 0u;
    if (search) {
        for (int t = sub; t < 9; t += G) {
            const int mx = cx + t % 3 - 1, my = cy + t / 3 - 1;
            if (mx < 0 || my < 0 || mx >= res || my >= res) continue;
            const int j = mx + my * res;
            if (j == i || !sc.fitPath(j)) continue;
            if (nav.reaches(x, nav.cellCentre(j))) bits |= 1u << t;
        }
    }
    for (int o = 1; o < G; o <<= 1) bits |= __shfl_xor_sync(0xffffffffu, bits, o);   // (aligned groups: partners inside)
    if (!search) return i;
    float best = 1e9f;
    int pick = i;
    for (int t = 0; t < 9; ++t) {
        const int mx = cx + t % 3 - 1, my = cy + t / 3 - 1;
        if (mx < 0 || my < 0 || mx >= res || my >= res) continue;
        const int j = mx + my * res;
        if (j == i || !sc.fitPath(j)) continue;
        const f2 q{g.x - (float(mx) + 0.5f), g.y - (float(my) + 0.5f)};
        const float d2 = q.x * q.x + q.y * q.y;
        if (d2 < best && (bits >> t & 1u)) { best = d2; pick = j; }
    }
    return pick;
}
#endif

struct Seated {
    const SwarmParams& P;
    const VenueArgs& V;

    __device__ __forceinline__ SeatedGeom geo() const { return SeatedGeom{V.seatDev}; }
    __device__ __forceinline__ StepUpConst stepUp() const { return StepUpConst{P.step_up_sample, P.step_up_tol, P.step_up_max_samples}; }
    __device__ __forceinline__ Stadium fence() const { return Stadium{P, V}; }   // the pitch fence and the router

    __device__ __forceinline__ float map(f3 p) const { return geo().sdfGrad(p).w; }             // cpu_crowd_sim.cpp:225-229
    __device__ __forceinline__ float4 mapExactGrad(f3 p) const { return geo().sdfGrad(p); }     // cpu_crowd_sim.cpp:239-242

    // cpu_crowd_sim.cpp:264-270: the heightfield's floor
    __device__ __forceinline__ bool floorUnderReach(f3 c, float zFrom, float down, float& zFloor) const {
        return geo().floorUnderReach(c, zFrom, down, P.body_radius, zFloor);
    }
    __device__ bool restOnFloor(f3& np, f3& nv, float zFrom) const {   // cpu_crowd_sim.cpp:317-325
        float zFloor;
        if (floorUnderReach(np, zFrom, P.body_radius, zFloor) && np.z < zFloor + P.body_radius) {
            np.z = zFloor + P.body_radius;
            nv.z = 0.0f;
            return true;
        }
        return false;
    }
    __device__ bool settleOnFloor(f3& np, f3& nv, float zFrom) const {   // cpu_crowd_sim.cpp:327-335
        float zFloor;
        if (floorUnderReach(np, zFrom, P.floor_settle_reach, zFloor)) {
            np.z = zFloor + P.body_radius;
            nv.z = 0.0f;
            return true;
        }
        return false;
    }

    // cpu_crowd_sim.cpp:299-315 calcGradient / sceneDist / sceneNormal
    __device__ f3 calcGradient(f3 p) const {
        const f3 kxyy{1.0f, -1.0f, -1.0f}, kyyx{-1.0f, -1.0f, 1.0f}, kyxy{-1.0f, 1.0f, -1.0f}, kxxx{1.0f, 1.0f, 1.0f};
        const float h = P.obstacle_grad_h;
        f3 a = kxyy * map(p + kxyy * h), b = kyyx * map(p + kyyx * h), c = kyxy * map(p + kyxy * h), d = kxxx * map(p + kxxx * h);
        return (a + b + c + d) * P.obstacle_grad_scale;
    }
    __device__ float sceneDist(f3 p, bool& fenceActive) const {
        const float dStadium = map(p);
        const float dFence = fence().sdFence(p) + P.body_radius;
        fenceActive = dFence < dStadium;
        return fenceActive ? dFence : dStadium;
    }
    __device__ f2 sceneNormal(f3 p, bool fenceActive) const {
        return fenceActive ? fence().sdFenceGradient(p) : xy(safeNormalize(calcGradient(p), P.safe_eps));
    }

    // cpu_crowd_sim.cpp:365-380 clearWalls, the analytic branch (the exact wall query, walls reaching the body's top)
    __device__ bool clearWalls(f3& np, f3& nv, f3& wall) const {
        bool moved = false;
        wall = f3{0.0f, 0.0f, 0.0f};
        const SwarmSeatedLayout& L = *V.seatDev;
        for (int pass = 0; pass < P.wall_passes; ++pass) {
            const f3 w = geo().wall(np + f3{0.0f, 0.0f, L.wall_above}, P.feeler_reach);
            if (w.z >= L.wall_clear) {
                if (w.z < WALL_NONE) wall = f3{w.x, w.y, w.z - L.wall_clear};
                break;
            }
            setXY(np, xy(np) + f2{w.x, w.y} * (L.wall_clear - w.z));
            moved = true;
            wall = f3{w.x, w.y, 0.0f};
            const float vDotN = dot(xy(nv), f2{w.x, w.y});
            if (vDotN < 0.0f) setXY(nv, xy(nv) - f2{w.x, w.y} * vDotN);
        }
        return moved;
    }
    // cpu_crowd_sim.cpp:423-427 wallPlaneProbe, the analytic branch
    __device__ f3 wallPlaneProbe(f3 np, float) const {
        const SwarmSeatedLayout& L = *V.seatDev;
        const f3 w = geo().wall(np + f3{0.0f, 0.0f, L.wall_above}, P.plane_probe_reach);
        return w.z >= 0.0f && w.z < WALL_NONE ? f3{w.x, w.y, smax(w.z - L.wall_clear, 0.0f)} : f3{0.0f, 0.0f, 0.0f};
    }

    __device__ __forceinline__ bool bakedSolid(f3 p) const { return fence().sdFence(p) >= 0.0f && mapExactGrad(p).w <= 0.0f; }

    // cpu_crowd_sim.cpp:449-463 sweepBack
    __device__ bool sweepBack(f3 pOld, f3& np, f3& nv) const {
        if (!bakedSolid(np)) return false;
        float lo = 0.0f, hi = 1.0f;
        if (!bakedSolid(f3{np.x, np.y, pOld.z})) lo = 1.0f;
        for (int i = 0; i < P.sweep_bisections; ++i) {
            const float t = 0.5f * (lo + hi);
            const f2 m = mix(xy(pOld), xy(np), t);
            if (bakedSolid(f3{m.x, m.y, pOld.z})) hi = t;
            else lo = t;
        }
        const f2 d = safeNormalize(xy(np) - xy(pOld), P.safe_eps);
        const f2 m = mix(xy(pOld), xy(np), lo);
        np = f3{m.x, m.y, pOld.z};
        const float vd = dot(xy(nv), d);
        if (vd > 0.0f) setXY(nv, xy(nv) - d * vd);
        nv.z = 0.0f;
        return true;
    }

    // cpu_crowd_sim.cpp:467-500 resolveStatic
    __device__ bool resolveStatic(f3 pOld, f3& np, f3& nv, bool settle, f3& wall, uint32_t& contact, float) const {
        const Stadium F = fence();
        if (F.fenceCCD(pOld, np, nv)) contact |= C_FENCE_CCD;
        const float dFence = F.sdFence(np);
        if (dFence < 0.0f) {
            const f2 n = F.sdFenceGradient(np);
            setXY(np, xy(np) - n * dFence);
            const float vDotN = dot(xy(nv), n);
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

    // cpu_crowd_sim.cpp:536-537 venueStepUpScan
    __device__ __forceinline__ float venueStepUpScan(f2 p0, f2 p1, float f0, f2& n) const {
        return geo().stepUpScan(stepUp(), p0, p1, f0, n);
    }

    // cpu_crowd_sim.cpp:601-617 venueBlockedWall, 622-650 venueEdgeMargin (out of line, on the geometry)
    __device__ __forceinline__ void venueBlockedWall(float f0, f3 pOld, f3& np, f3& nv) const {
        geo().blockedWall(stepUp(), P.feeler_reach, P.body_radius, P.floor_settle_reach, f0, pOld, np, nv);
    }
    __device__ __forceinline__ void venueEdgeMargin(f3 pOld, float f0, f3& np, f3& nv) const {
        geo().edgeMargin(stepUp(), P.body_radius, P.floor_settle_reach, pOld, f0, np, nv);
    }

    // cpu_crowd_sim.cpp:566-597 limitStepUp, the analytic branch
    __device__ bool limitStepUp(f3 pOld, f3& np, f3& nv, float) const {
        float f0;
        if (!floorUnderReach(pOld, pOld.z, P.step_up_floor_reach, f0)) f0 = pOld.z - P.step_up_floor_reach;
        f2 n;
        const float t = venueStepUpScan(xy(pOld), xy(np), f0, n);
        if (t >= 1.0f) {
            venueEdgeMargin(pOld, f0, np, nv);
            return false;
        }
        f2 q = mix(xy(pOld), xy(np), t);
        const f2 rest = xy(np) - q;
        const f2 tangent = rest - n * dot(rest, n);
        const float lt = length(tangent);
        if (lt > 0.0f) {
            for (int k = 0; k < P.step_up_slide_tries; ++k) {
                const f2 slide = q + tangent * P.step_up_slide[k][0] + n * (lt * P.step_up_slide[k][1]);
                f2 n2;
                if (fence().sdFence(f3{slide.x, slide.y, 0.0f}) >= 0.0f && venueStepUpScan(q, slide, f0, n2) >= 1.0f) { q = slide; break; }
            }
        }
        const float vn = dot(xy(nv), n);
        if (vn < 0.0f) setXY(nv, xy(nv) - n * vn);
        float zFloor;
        if (floorUnderReach(f3{q.x, q.y, pOld.z}, pOld.z, P.floor_settle_reach, zFloor)) {
            np = f3{q.x, q.y, zFloor + P.body_radius};
            nv.z = 0.0f;
        } else {
            np = f3{q.x, q.y, smin(np.z, pOld.z)};
        }
        venueBlockedWall(f0, pOld, np, nv);
        venueEdgeMargin(pOld, f0, np, nv);
        return true;
    }

    // e_goal: the navigation field's anchor lookup; without a field, the egress router (cpu_crowd_sim.cpp:213-218)
    __device__ __forceinline__ f2 goal(f3 p) const {
        if (!V.navCells) return fence().goal(p);
        return SeatedNav{geo(), stepUp(), P.goal_deadzone, P.feeler_reach, P.safe_eps, V.navCells, V.navRes, V.navOrigin,
                         V.navCell, V.navInv}.goal(p);
    }
    // e_goal under the queue-aware exit choice: the assigned exit's anchor in the agent's choice cell
    // (cpu_crowd_sim.cpp:214, nav::choiceGoal)
    __device__ __forceinline__ f2 choiceGoalCell(f3 p, uint32_t exit, int cell) const {
        return SeatedChoice{SeatedNav{geo(), stepUp(), P.goal_deadzone, P.feeler_reach, P.safe_eps, nullptr, V.navRes,
                                      V.navOrigin, V.navCell, V.navInv},
                            V.choiceIndex, V.choiceEntries}.goalFromCell(p, exit, cell);
    }
    __device__ __forceinline__ f2 choiceGoal(f3 p, uint32_t exit) const {
        return SeatedChoice{SeatedNav{geo(), stepUp(), P.goal_deadzone, P.feeler_reach, P.safe_eps, nullptr, V.navRes,
                                      V.navOrigin, V.navCell, V.navInv},
                            V.choiceIndex, V.choiceEntries}.goal(p, exit);
    }

    __device__ __forceinline__ bool exits(float4 p) const { return fence().exits(p); }   // cpu_crowd_sim.cpp:662-668
    __device__ __forceinline__ void fenceProject(f3& q) const { fence().fenceProject(q); }
    __device__ __forceinline__ float speedFactor(f3) const { return 1.0f; }

    // physics.comp inclineFreeSpeed / inclineHeadwayTime (venue.cpp:652-670): smoothstep blends by the slope
    __device__ __forceinline__ float inclineBlend(float g) const {
        const float u = sclamp(fabsf(g) * P.incline_inv_ref_slope, 0.0f, 1.0f);
        const float uu = u * u, w = 3.0f - 2.0f * u;
        return uu * w;
    }
    __device__ __forceinline__ float inclineFreeSpeed(float g) const {
        const float t = inclineBlend(g);
        const float vStair = g > 0.0f ? P.v_stair_up : P.v_stair_down;
        const float dv = vStair - P.v_max;
        const float k = dv * t;
        return P.v_max + k;
    }
    __device__ __forceinline__ float inclineHeadwayTime(float g) const {
        const float t = inclineBlend(g);
        const float tStair = g > 0.0f ? V.stairTUp : V.stairTDown;
        const float dt = tStair - P.t_headway;
        const float k = dt * t;
        return P.t_headway + k;
    }
    // cpu_crowd_sim.cpp:727-733: the desired speed of the headway rule with the incline speed and stair spacing
    __device__ float desiredSpeed(f2 pxy, f2 eGoal, float sAhead) const {
        const float slope = V.incline ? geo().floorSlope(pxy, eGoal) : 0.0f;
        const float vFree = V.incline ? inclineFreeSpeed(slope) : P.v_max;
        const float v = V.stairHw && slope != 0.0f
                            ? sclamp((sAhead - P.body_diam) / inclineHeadwayTime(slope), 0.0f, vFree)
                            : sclamp((sAhead - P.body_diam) * P.headway_rate, 0.0f, vFree);
        return v * length(eGoal);
    }
    // the longest headway time gap any slope gives (the predict pass's search disk)
    __device__ __forceinline__ float maxHeadwayTime() const {
        const float t0 = 1.0f / P.headway_rate;
        return V.stairHw ? smax(t0, smax(V.stairTUp, V.stairTDown)) * 1.001f : t0;
    }
};

}  // namespace swarm_gpu
