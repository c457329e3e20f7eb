// Tile-shape autotuner for the FCT sub-step kernels.
//
// Every FCT kernel walks a list of tiles, one thread block per tile of tile_j (p, the
// coalesced axis) x tile_i (x) cells.  The best shape depends on the patch sizes of the
// set (ragged edges, occupancy, register pressure of the precision's kernels), so the
// engine measures it: for each candidate the tile list is rebuilt and the sub-steps that
// leave the solution unchanged between steps (gamma, faces, fluxes, ds/f2, limiter R and
// C — their outputs are recomputed before being read in the next step) are timed with CUDA
// events on the engine's stream; the fastest shape is kept for the set and becomes the
// default for new sets of the same precision.  The tile shape changes no arithmetic.
#include <array>

#include "engine.hpp"

namespace vx {

std::pair<int, int> Engine::autotune(const std::vector<Run *> &set, int reps) {
    static const int kShapes64[][2] = {{32, 4}, {32, 8}, {32, 16}, {64, 4}, {64, 8}, {128, 2}, {128, 4}};
    // FP32: 128 p cells (four per thread) by 1 .. 16 rows
    static const int kShapes32[][2] = {{128, 1}, {128, 2}, {128, 4}, {128, 8}, {128, 16}};
    LaunchSet &L = get_set(set);
    FctLaunch fl{};
    fl.patches = L.dpatch.p;
    fl.fields = L.dfields.as<RunFields>();
    fl.params = L.dparams.as<double>();
    fl.params32 = L.dparams32.as<float>();
    fl.step = 0;
    fl.stream = stream;
    auto run_subs = [&]() {
        if (L.precision == kF32)
            for (int sub : {kSubXFlux, kSubPFlux, kSubDsF2, kSubLimR, kSubLimC}) launch_fct32_substep(fl, sub);
        else
            for (int sub : {kSubGamma, kSubFaces, kSubFlux, kSubDsF2, kSubLimR, kSubLimC}) launch_fct64_substep(fl, sub);
    };
    double best_ms = 1e300;
    int best[2] = {L.tile_j, L.tile_i};
    std::vector<std::array<int, 2>> shapes;
    if (L.precision == kF32)
        for (auto &sh : kShapes32) shapes.push_back({sh[0], sh[1]});
    else
        for (auto &sh : kShapes64) shapes.push_back({sh[0], sh[1]});
    for (auto &sh : shapes) {
        L.tile_j = sh[0];
        L.tile_i = sh[1];
        build_tiles(L);  // reallocates every tile list: take the pointers afresh
        fl.tiles = L.dtiles.as<TileRef>();
        fl.ntiles = L.ntiles;
        fl.xtiles = L.dxtiles.as<TileRef>();
        fl.ptiles = L.dptiles.as<TileRef>();
        fl.nxtiles = L.nxtiles;
        fl.nptiles = L.nptiles;
        fl.tile_j = L.tile_j;
        fl.tile_i = L.tile_i;
        run_subs();  // warm-up
        if (cudaGetLastError() != cudaSuccess) continue;  // shape not launchable here
        timer_begin();
        for (int r = 0; r < reps; r++) run_subs();
        const double ms = timer_end() / reps;
        kernel_launches += (L.precision == kF32 ? 5 : 6) * (reps + 1);
        if (ms < best_ms) {
            best_ms = ms;
            best[0] = sh[0];
            best[1] = sh[1];
        }
    }
    L.tile_j = best[0];
    L.tile_i = best[1];
    build_tiles(L);
    if (L.graph) {  // the captured step holds the old tile list
        cudaGraphExecDestroy(L.graph);
        L.graph = nullptr;
    }
    tile_pref[L.precision == kF32][0] = best[0];
    tile_pref[L.precision == kF32][1] = best[1];
    sync();
    return {best[0], best[1]};
}

}  // namespace vx
