// Field-side kernels of the FP32 precision form: the moments kernel over the bodies of
// moments32.cuh (one warp per coarse column) and the per-cell A^2 copy.
#include <cuda_runtime.h>

#include "moments32.cuh"

namespace vx {

__global__ void k32_moments(MomLaunch M) {
    VX_PDL_WAIT();
    if (M.asq32)
        for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < M.nruns * (M.maxnf + 1); e += gridDim.x * blockDim.x)
            asq32_copy(M, e);
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= M.ncols) return;
    moments32_column(M, warp, threadIdx.x & 31);
}

__global__ void k_acell32(const RunFields *fields, int nruns) {
    VX_PDL_WAIT();
    const int run = blockIdx.y;
    if (run >= nruns) return;
    acell32_cell(fields, run, blockIdx.x * blockDim.x + threadIdx.x);
}

void launch_moments32(const MomLaunch &M) {
    if (M.ncols == 0) return;
    if (M.acell) vx_launch(k_acell32, dim3((M.maxnf + 255) / 256, M.nruns), 256, 0, M.stream, M.fields, M.nruns);
    const int threads = 256;
    const int blocks = (M.ncols * 32 + threads - 1) / threads;
    vx_launch(k32_moments, blocks, threads, 0, M.stream, M);
}

}  // namespace vx
