// Test infrastructure only: the product's seated-venue geometry and navigation lookup (csrc/venue_seated.cuh) compiled
// for the host, so that a CPU test compares them point by point with the reference's own functions (seated::*,
// nav::goal) through oracle/_ref. The same source compiles into the CUDA step; -ffp-contract=off here as there.
#include "../swarm-crowd-simulation_gb300/csrc/venue_seated.cuh"

using namespace swarm_gpu;

// op 0 floorHeight(x, y) -> 1 | 1 cellKey(x, y) -> 2 | 2 sdfGrad(x, y, z) -> 4 | 3 wall(x, y, z, reach) -> 3 |
// 4 stepUpScan(x0, y0, x1, y1, f0) -> (t, n.x, n.y) | 5 floorSlope(x, y, ex, ey) -> 1 | 6 nav goal(x, y, z) -> 2
extern "C" int hs_eval(const SwarmSeatedLayout* L, const SwarmParams* P, int op, int n, const float* in, float* out,
                       const float* nav, int navRes, float navOrigin, float navCell, float navInv) {
    const std::vector<unsigned char> blob = seatedBlob(*L);   // the layout and its tables, as the step holds them
    const SeatedGeom G{reinterpret_cast<const SwarmSeatedLayout*>(blob.data())};
    for (int i = 0; i < n; ++i) {
        switch (op) {
        case 0: out[i] = G.floorHeight(f2{in[2 * i], in[2 * i + 1]}); break;
        case 1: { const f2 k = G.cellKey(f2{in[2 * i], in[2 * i + 1]}); out[2 * i] = k.x; out[2 * i + 1] = k.y; break; }
        case 2: {
            const float4 g = G.sdfGrad(f3{in[3 * i], in[3 * i + 1], in[3 * i + 2]});
            out[4 * i] = g.x; out[4 * i + 1] = g.y; out[4 * i + 2] = g.z; out[4 * i + 3] = g.w;
            break;
        }
        case 3: {
            const f3 w = G.wall(f3{in[4 * i], in[4 * i + 1], in[4 * i + 2]}, in[4 * i + 3]);
            out[3 * i] = w.x; out[3 * i + 1] = w.y; out[3 * i + 2] = w.z;
            break;
        }
        case 4: {
            f2 nn;
            const float t = G.stepUpScan(StepUpConst{P->step_up_sample, P->step_up_tol, P->step_up_max_samples}, f2{in[5 * i], in[5 * i + 1]}, f2{in[5 * i + 2], in[5 * i + 3]}, in[5 * i + 4], nn);
            out[3 * i] = t; out[3 * i + 1] = nn.x; out[3 * i + 2] = nn.y;
            break;
        }
        case 5: out[i] = G.floorSlope(f2{in[4 * i], in[4 * i + 1]}, f2{in[4 * i + 2], in[4 * i + 3]}); break;
        case 6: {
            const SeatedNav N{G, StepUpConst{P->step_up_sample, P->step_up_tol, P->step_up_max_samples}, P->goal_deadzone,
                               P->feeler_reach, P->safe_eps, reinterpret_cast<const float4*>(nav), navRes, navOrigin, navCell, navInv};
            const f2 e = N.goal(f3{in[3 * i], in[3 * i + 1], in[3 * i + 2]});
            out[2 * i] = e.x; out[2 * i + 1] = e.y;
            break;
        }
        default: return -1;
        }
    }
    return 0;
}
