// FP32 precision form of the FCT sub-steps as one kernel per sub-step (the bodies are in
// fct32.cuh, shared with the persistent stage kernel of stage32.cu).
// Compiled with fused multiply-add allowed.
#include <cuda_runtime.h>

#include "fct32.cuh"

namespace vx {

// Streaming sub-steps: one block of (32, tile_i) threads per tile.
__global__ void k32_ds_f2(const P32 *patches, const TileRef *tiles, const float *params, int s) {
    VX_PDL_WAIT();
    ds_f2_32(patches, tiles[blockIdx.x], (int)threadIdx.x, (int)threadIdx.y, params, s);
}
__global__ void k32_limR(const P32 *patches, const TileRef *tiles) {
    VX_PDL_WAIT();
    limR32(patches, tiles[blockIdx.x], (int)threadIdx.x, (int)threadIdx.y);
}
__global__ void k32_limC(const P32 *patches, const TileRef *tiles) {
    VX_PDL_WAIT();
    limC32(patches, tiles[blockIdx.x], (int)threadIdx.x, (int)threadIdx.y);
}
__global__ void k32_update(const P32 *patches, const TileRef *tiles) {
    VX_PDL_WAIT();
    update32(patches, tiles[blockIdx.x], (int)threadIdx.x, (int)threadIdx.y);
}
__global__ void k32_copy10(const P32 *patches, const TileRef *tiles) {
    VX_PDL_WAIT();
    copy10_32(patches, tiles[blockIdx.x], (int)threadIdx.x, (int)threadIdx.y);
}

// Fused face + flux sub-steps: one warp per strip tile (whole warps leave together).
__global__ void k32_xflux(const P32 *patches, const TileRef *tiles, int ntiles, const RunFields *fields, int step,
                          int use_f0) {
    VX_PDL_WAIT();
    const int wt = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (wt >= ntiles) return;
    xflux32(patches, tiles[wt], threadIdx.x & 31, fields, step, use_f0);
}
__global__ void k32_pflux(const P32 *patches, const TileRef *tiles, int ntiles, const RunFields *fields, int step,
                          int use_f0) {
    VX_PDL_WAIT();
    const int wt = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (wt >= ntiles) return;
    pflux32(patches, tiles[wt], threadIdx.x & 31, fields, step, use_f0);
}

void launch_fct32_substep(const FctLaunch &L, int sub) {
    // streaming kernels: tiles of tile_i rows x 128 p cells, four cells per thread
    dim3 blk(32, L.tile_i ? L.tile_i : 8);
    const P32 *pp = (const P32 *)L.patches;
    if (L.ntiles == 0) return;
    switch (sub) {
        case kSubDsF2:
            vx_launch(k32_ds_f2, L.ntiles, blk, 0, L.stream, pp, L.tiles, L.params32, L.step);
            break;
        case kSubLimR:
            vx_launch(k32_limR, L.ntiles, blk, 0, L.stream, pp, L.tiles);
            break;
        case kSubLimC:
            vx_launch(k32_limC, L.ntiles, blk, 0, L.stream, pp, L.tiles);
            break;
        case kSubUpdate:
            vx_launch(k32_update, L.ntiles, blk, 0, L.stream, pp, L.tiles);
            break;
        case kSubCopy10:
            vx_launch(k32_copy10, L.ntiles, blk, 0, L.stream, pp, L.tiles);
            break;
        case kSubXFlux:
            if (L.nxtiles) vx_launch(k32_xflux, (L.nxtiles + 3) / 4, 128, 0, L.stream, pp, L.xtiles, L.nxtiles, L.fields, L.step, L.use_f0);
            break;
        case kSubPFlux:
            if (L.nptiles) vx_launch(k32_pflux, (L.nptiles + 3) / 4, 128, 0, L.stream, pp, L.ptiles, L.nptiles, L.fields, L.step, L.use_f0);
            break;
        default:  // the FP32 form has no separate gamma / face / flux sub-steps (fused above)
            break;
    }
}

}  // namespace vx
