// CFL time-step bound for callers that must not allocate device memory.
//
// Some callers cannot call cudaMalloc: an adaptive time-step controller that polls the
// bound between steps of a solver whose device memory is committed up front (a serving
// process that handed its whole budget to resident solves, or an embedding application
// with a fixed memory plan), and any caller that must not trigger the device-wide
// synchronisation that cudaMalloc / cudaFree may imply while other streams run.
// vx_cfl_bound_noalloc computes the same bound as vx_run_calculate_dt
// (EMFieldSolver::EstimateCFLBound, EMSolver.cpp:631-664) from field arrays the caller
// already has on the device.  Its only scratch memory — one partial maximum per block of
// 256 cells — is the file-scope array below, so it allocates nothing.
//
// The scratch is shared by every call on a device and keeps the last call's contents;
// each call writes every entry it later reads, so nothing needs clearing, but calls that
// overlap on the GPU (several host threads, or several streams at once) race on it.
// Every GPU that loads the library holds the array until the process exits.
//
// Compiled with --fmad=false: the arithmetic is that of the run's own CFL kernel, so the
// result equals vx_run_calculate_dt's bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

#include "../../include/vx.h"
#include "vx_common.hpp"

namespace vx {

void set_last_error(const std::string &msg);

namespace {

constexpr int kCflThreads = 256;
constexpr int kCflMaxBlocks = VX_CFL_NOALLOC_MAX_CELLS / kCflThreads;

__device__ __align__(256) double cfl_scratch[kCflMaxBlocks];

struct CflSpecies {
    double aq[8], m[8], dps[8];
    double dps_max;
    int ns;
};

__global__ void k_cfl_partial(const double *Ay, const double *Az, const double *By, const double *Bz,
                              const double *Ex, int n, CflSpecies S, double *partial) {
    __shared__ double red[kCflThreads];
    const int i = blockIdx.x * kCflThreads + threadIdx.x;
    double pc = 0.0;
    if (i < n) {
        double Azv = Az[i], Ayv = Ay[i];
        double As = Ayv * Ayv + Azv * Azv;
        double temp = 0.0;
        for (int j = 0; j < S.ns; j++) {
            double aq = S.aq[j], m = S.m[j], dps = S.dps[j];
            double v = aq / m / sqrt(1 + As / ((m * kCs) * (m * kCs))) * dps;
            temp = (temp < v) ? v : temp;
        }
        pc = temp * fabs(Ayv * Bz[i] - Azv * By[i]) + S.dps_max * fabs(Ex[i]);
    }
    red[threadIdx.x] = pc;
    __syncthreads();
    for (int s = kCflThreads / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            double o = red[threadIdx.x + s];
            red[threadIdx.x] = (red[threadIdx.x] < o) ? o : red[threadIdx.x];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// Folds the partial maxima into partial[0].
__global__ void k_cfl_fold(double *partial, int blocks) {
    __shared__ double red[kCflThreads];
    double v = 0.0;
    for (int b = threadIdx.x; b < blocks; b += kCflThreads) v = (v < partial[b]) ? partial[b] : v;
    red[threadIdx.x] = v;
    __syncthreads();
    for (int s = kCflThreads / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            double o = red[threadIdx.x + s];
            red[threadIdx.x] = (red[threadIdx.x] < o) ? o : red[threadIdx.x];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[0] = red[0];
}

// Device address of the scratch array, looked up once per device with that device
// current (host code only sees a stand-in for the symbol, not a device address).  The
// address is kept for the life of the process: after cudaDeviceReset the module is
// loaded again and the array may move, so the entry point must not be used on a device
// that has been reset.
double *scratch_on_current_device(int *err) {
    static std::mutex mu;
    static double *addr[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        *err = 1;
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, cfl_scratch) != cudaSuccess || !p) {
            *err = 2;
            return nullptr;
        }
        addr[dev] = (double *)p;
    }
    *err = 0;
    return addr[dev];
}

}  // namespace
}  // namespace vx

extern "C" int vx_cfl_bound_noalloc(const double *Ay, const double *Az, const double *By, const double *Bz,
                                    const double *Ex, int n, const double *q, const double *m, const double *dp0,
                                    int nspecies, double dx0, double cfl, void *stream, double *dt) {
    using namespace vx;
    if (!Ay || !Az || !By || !Bz || !Ex || !q || !m || !dp0 || !dt || n <= 0 || nspecies <= 0 || nspecies > 8 ||
        !(dx0 > 0)) {
        set_last_error("vx_cfl_bound_noalloc: bad argument");
        return VX_ERR_INVALID;
    }
    for (int i = 0; i < nspecies; i++) {
        if (!(std::isfinite(dp0[i]) && dp0[i] > 0) || !(std::isfinite(m[i]) && m[i] > 0) || !std::isfinite(q[i])) {
            set_last_error("vx_cfl_bound_noalloc: species " + std::to_string(i) +
                           " needs a finite positive dp0 and mass and a finite charge");
            return VX_ERR_INVALID;
        }
    }
    if (n > VX_CFL_NOALLOC_MAX_CELLS) {
        set_last_error("vx_cfl_bound_noalloc: n = " + std::to_string(n) + " exceeds the limit of " +
                       std::to_string(VX_CFL_NOALLOC_MAX_CELLS) + " finest cells (its scratch is a fixed array)");
        return VX_ERR_INVALID;
    }
    // an error the caller left pending is reported as such, not blamed on this call
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("vx_cfl_bound_noalloc: a CUDA error was pending before the call: ") +
                       cudaGetErrorString(e));
        return VX_ERR_CUDA;
    }
    int err = 0;
    double *partial = scratch_on_current_device(&err);
    if (!partial) {
        set_last_error(err == 2 ? "vx_cfl_bound_noalloc: cudaGetSymbolAddress failed"
                                : "vx_cfl_bound_noalloc: no current CUDA device");
        return VX_ERR_CUDA;
    }
    // the species table of EMSolver.cpp:631-646, built as the run's launch set builds it
    CflSpecies S{};
    S.ns = nspecies;
    double dps_max(0.0);
    for (int i = 0; i < nspecies; i++) {
        double dps = 1 / dp0[i];
        dps_max = std::max(dps_max, std::fabs(q[i]) * dps);
        S.aq[i] = std::fabs(q[i]);
        S.m[i] = m[i];
        S.dps[i] = dps;
    }
    S.dps_max = dps_max;
    cudaStream_t st = (cudaStream_t)stream;
    const int blocks = (n + kCflThreads - 1) / kCflThreads;
    k_cfl_partial<<<blocks, kCflThreads, 0, st>>>(Ay, Az, By, Bz, Ex, n, S, partial);
    e = cudaGetLastError();
    if (e == cudaSuccess) {
        k_cfl_fold<<<1, kCflThreads, 0, st>>>(partial, blocks);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        set_last_error(std::string("vx_cfl_bound_noalloc: launch failed: ") + cudaGetErrorString(e));
        return VX_ERR_CUDA;
    }
    double pc = 0.0;
    e = cudaMemcpyAsync(&pc, partial, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_last_error(std::string("vx_cfl_bound_noalloc: ") + cudaGetErrorString(e));
        return VX_ERR_CUDA;
    }
    double bound = 1.0 / std::max((kCs / dx0 + pc), 1e-40);
    *dt = cfl * bound;
    return VX_OK;
}
