// FP32 launch sets: the persistent stage kernels and the per-sub-step kernels of the op
// batches, assembly and Maxwell stage.
//
// A persistent stage kernel runs a whole run of phases of one RK stage (Mesh::Advance ->
// Level::FCTTimeStep and EMFieldSolver::RGKStep for every patch of every run of the set,
// Mesh.cpp:64-89, EMSolver.cpp:194-202) in one cooperative launch: every block walks each
// phase's work list (tiles, strips, columns, cells, ops) with a grid stride, and a
// grid-wide barrier separates phases that read what the previous one wrote.  The work of
// a phase is the same body, in the same translation unit configuration (fused
// multiply-add allowed), as the per-sub-step kernel that does it in the graph form
// (fct32.cu, fields32.cu, and the kernels below), so both forms give the same bits.
//
// Phases independent of each other share a barrier interval: the x fluxes run beside the
// moments (before the Poisson solve: they read neither rho nor E_x), and the Maxwell stage
// (which reads J and writes A, E, B and a^2, none of which the FP32 FCT phases read — they
// read the FP32 copies of a^2 and E_x) runs its three steps beside the p flux, ds/f2 and
// limiter R phases; its last step also writes the FP32 a^2 copy for the next stage.
#include <cuda_runtime.h>

#include <algorithm>

#include "amr_ops.cuh"
#include "fct32.cuh"
#include "field_ops.cuh"
#include "moments32.cuh"

namespace vx {

constexpr int kStageThreads = 256;  // 8 warps: one (32, 8) tile row set, eight strips or columns
constexpr unsigned kMaxPolls = 1u << 25;  // second bound of a barrier wait (>= 64 ns each)

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_relaxed_s32(const int *p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid-wide barrier of a cooperative launch with a bounded wait (see GridSyncState).
// Arrivals only grow during a launch: barrier k is complete at k * expected arrivals, and
// the block that makes that arrival publishes k in `released`, which the others poll.
struct GridBarrier {
    GridSyncState *st;
    unsigned expected, target;
    unsigned long long limit_ns;
    int index;
    unsigned long long *trace;
    __device__ GridBarrier(GridSyncState *s, unsigned long long lim, unsigned exp, unsigned long long *tr)
        : st(s), expected(exp), target(0), limit_ns(lim), index(0), trace(tr) {
        if (trace && blockIdx.x == 0 && threadIdx.x == 0) trace[0] = global_ns();
    }
    __device__ void sync() {
        __syncthreads();  // the block's writes of the phase are done
        target += expected;
        index++;
        if (threadIdx.x == 0) {
            if (trace && 2 * index < kStageTraceSlots) atomicMax(&trace[2 * index - 1], global_ns());
            __threadfence();  // ... and visible device-wide before the arrival
            if (atomicAdd(&st->arrive, 1u) + 1 == target) {
                atomicExch(&st->next, 0u);  // no block takes work of the finished phase any more
                __threadfence();  // cumulative: every arrival's writes before the release
                atomicMax(&st->released, (unsigned)index);  // the last arrival releases the rest
            } else if (ld_relaxed_s32(&st->err) == 0) {
                const unsigned long long t0 = global_ns();
                for (unsigned poll = 0;; poll++) {
                    if (ld_acquire_u32(&st->released) >= (unsigned)index) break;
                    if ((poll & 63u) == 63u && ld_relaxed_s32(&st->err) != 0) break;  // another block gave up
                    if (poll >= kMaxPolls || global_ns() - t0 > limit_ns) {
                        atomicCAS(&st->err, 0, index);
                        break;
                    }
                    __nanosleep(64);
                }
            }
            __threadfence();  // the other blocks' phase writes are seen by this block's loads
            if (trace && blockIdx.x == 0 && 2 * index < kStageTraceSlots) trace[2 * index] = global_ns();
        }
        __syncthreads();
    }
    // The last block to leave resets the arrival counts for the next launch on the stream.
    __device__ void finish() {
        __syncthreads();
        if (threadIdx.x == 0) {
            if (trace && 2 * index + 1 < kStageTraceSlots) atomicMax(&trace[2 * index + 1], global_ns());
            __threadfence();
            if (atomicAdd(&st->leave, 1u) + 1 == gridDim.x) {
                atomicExch(&st->arrive, 0u);
                atomicExch(&st->released, 0u);
                atomicExch(&st->next, 0u);
                atomicExch(&st->leave, 0u);
                __threadfence();
            }
        }
    }
};

// The tiles of a streaming phase (tile_i rows x 128 p cells, a power of two of rows):
// a block's 8 warps take 8 / tile_i tiles at a time, or walk a taller tile 8 rows at a time.
template <class Body>
__device__ __forceinline__ void for_tiles(const FctLaunch &F, Body body) {
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int ti = F.tile_i > 0 ? F.tile_i : 8;
    if (ti >= 8) {
        for (int t = blockIdx.x; t < F.ntiles; t += gridDim.x)
            for (int r = ty; r < ti; r += 8) body(F.tiles[t], tx, r);
    } else {
        const int per = 8 / ti;
        if (ty >= per * ti) return;  // warps left over by a tile height that does not divide 8
        for (int t0 = blockIdx.x * per; t0 < F.ntiles; t0 += gridDim.x * per) {
            const int t = t0 + ty / ti;
            if (t < F.ntiles) body(F.tiles[t], tx, ty % ti);
        }
    }
}

// Cells or ops e of a phase in runs of 32 (one warp, coalesced), the runs dealt
// round-robin over the blocks: the few heavy items of a small field grid or op batch are
// spread over every SM instead of landing on the first blocks, which also carry their
// share of the tiles.
template <class Body>
__device__ __forceinline__ void for_cells(long long n, Body body) {
    const long long nt = (long long)gridDim.x * kStageThreads;
    const long long e0 = ((long long)(threadIdx.x >> 5) * gridDim.x + blockIdx.x) * 32 + (threadIdx.x & 31);
    for (long long e = e0; e < n; e += nt) body(e);
}

// Warp-sized work units [0, n) (flux strips, moment columns) taken from the phase's
// counter, `chunk` at a time: a warp that finishes early takes more, so a phase with about
// as many units as warps ends after one unit's time, not two.  Whole warps call it.
template <class Body>
__device__ __forceinline__ void for_warp_units(GridSyncState *st, int n, Body body) {
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (kStageThreads / 32);
    const int chunk = max(1, min(16, n / (8 * warps)));
    for (;;) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(&st->next, (unsigned)chunk);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= (unsigned)n) break;
        const int end = min(n, (int)base + chunk);
        for (int u = (int)base; u < end; u++) body(u);
    }
}

// [per-cell A^2 copy] | FP32 moments + the a^2 copy | assembly of rho and J.
__global__ void __launch_bounds__(kStageThreads, 5) k32_stage_pre(Stage32Launch L) {
    GridBarrier bar(L.sync, L.limit_ns, gridDim.x + (unsigned)L.phantom, L.trace);
    const MomLaunch &M = L.ml;
    const int lane = threadIdx.x & 31;
    if (M.acell) {  // stage 0: the FP32 copies of the per-cell A^2 and of a^2
        for_cells((long long)M.nruns * M.maxnf, [&](long long e) {
            acell32_cell(M.fields, (int)(e / M.maxnf), (int)(e % M.maxnf));
        });
        for_cells((long long)M.nruns * (M.maxnf + 1), [&](long long e) { asq32_copy(M, (int)e); });
        bar.sync();
    }
    // moments (longest columns first) | x fluxes (Rectangle.cpp:1255-1325; they read f and
    // the a^2 copy): one queue of warp units, the columns, then the strips
    const FctLaunch &F = L.fl;
    const P32 *patches = (const P32 *)F.patches;
    for_warp_units(L.sync, M.ncols + F.nxtiles, [&](int u) {
        if (u < M.ncols) moments32_column(M, u, lane);
        else xflux32(patches, F.xtiles[u - M.ncols], lane, F.fields, L.step, F.use_f0);
    });
    bar.sync();
    const AsmLaunch &A = L.al;
    for_cells((long long)A.nruns * A.maxn, [&](long long e) { assemble_cell(A, (int)(e / A.maxn), (int)(e % A.maxn)); });
    bar.finish();
}

// The ops of batch b, round-robin over the blocks.
template <class Body>
__device__ __forceinline__ void for_ops(const int *ptr, int b, Body body) {
    const int lo = ptr[b], hi = ptr[b + 1];
    for_cells(hi - lo, [&](long long e) { body(lo + (int)e); });
}

// The FCT stage of every patch (fluxes .. ghost fills of f1) with the Maxwell stage beside it.
// Five blocks per SM (48 registers, a few spilled on the limiter and interpolation paths):
// the p-flux strips and streaming phases gain more from the extra warps than the spills
// cost (64-run ensemble 79.8 -> 77.4 ms per step, 4096 x 512 case 1.90 -> 1.85 ms).
__global__ void __launch_bounds__(kStageThreads, 5) k32_stage_fct(Stage32Launch L) {
    GridBarrier bar(L.sync, L.limit_ns, gridDim.x + (unsigned)L.phantom, L.trace);
    const FctLaunch &F = L.fl;
    const P32 *patches = (const P32 *)F.patches;
    const int s = L.step;
    const int lane = threadIdx.x & 31;
    const MaxwellLaunch &X = L.mx;
    const long long mxn = (long long)X.nruns * X.maxnf;
    // p fluxes (Rectangle.cpp:1326-1394; E_x from the solve) | Maxwell right-hand side
    for_cells(mxn, [&](long long e) { mx_rhs_cell(X, (int)(e / X.maxnf), (int)(e % X.maxnf)); });
    for_warp_units(L.sync, F.nptiles, [&](int w) { pflux32(patches, F.ptiles[w], lane, F.fields, s, F.use_f0); });
    bar.sync();
    // coarse faces on coarse/fine interfaces, batch by batch
    for (int b = 0; b < L.niface_b; b++) {
        for_ops(L.iface_ptr, b, [&](int k) { iface_op(patches, L.iface, k, s); });
        bar.sync();
    }
    // RK flux combination and low-order solution | Maxwell stage combination
    for_tiles(F, [&](const TileRef &t, int tx, int row) { ds_f2_32(patches, t, tx, row, F.params32, s); });
    for_cells(mxn, [&](long long e) { mx_update_cell(X, (int)(e / X.maxnf), (int)(e % X.maxnf)); });
    bar.sync();
    // ghost cells of f2 (Mesh::PushData(2))
    for (int b = 0; b < L.nghost_b; b++) {
        for_ops(L.ghost_ptr, b, [&](int k) { ghost_op(patches, L.ghost, k, 2); });
        bar.sync();
    }
    // limiter R | a^2 on the faces
    for_tiles(F, [&](const TileRef &t, int tx, int row) { limR32(patches, t, tx, row); });
    for_cells(mxn, [&](long long e) { mx_asq_cell(X, (int)(e / X.maxnf), (int)(e % X.maxnf)); });
    bar.sync();
    // limiter C, then its exchange across patch edges (Mesh::PushBoundaryC), batch by batch
    for_tiles(F, [&](const TileRef &t, int tx, int row) { limC32(patches, t, tx, row); });
    bar.sync();
    for (int b = 0; b < L.ncsync_b; b++) {
        for_ops(L.csync_ptr, b, [&](int k) { csync_op(patches, L.csync, k); });
        bar.sync();
    }
    // antidiffusive update, then the ghost cells of f1 (Mesh::PushData(1))
    for_tiles(F, [&](const TileRef &t, int tx, int row) { update32(patches, t, tx, row); });
    bar.sync();
    for (int b = 0; b < L.nghost_b; b++) {
        for_ops(L.ghost_ptr, b, [&](int k) { ghost_op(patches, L.ghost, k, 1); });
        if (b + 1 < L.nghost_b || s == 5) bar.sync();
    }
    if (s == 5)  // FCTTimeStep(.., 3) at the last stage: f0 = f1
        for_tiles(F, [&](const TileRef &t, int tx, int row) { copy10_32(patches, t, tx, row); });
    bar.finish();
}

static int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

int stage32_grid_limit(int which_fct) {
    static int limit[2] = {0, 0};
    int &lim = limit[which_fct ? 1 : 0];
    if (!lim) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (which_fct) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k32_stage_fct, kStageThreads, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k32_stage_pre, kStageThreads, 0);
        lim = std::max(1, sms * per);
    }
    return lim;
}

template <class K>
static void launch_coop(K kernel, int blocks, const Stage32Launch &L) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(kStageThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = L.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;  // all blocks co-resident, or the launch fails
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, L);  // errors surface through cudaGetLastError
}

void launch_stage32_pre(const Stage32Launch &L) {
    const MomLaunch &M = L.ml;
    int need = std::max({cdiv(M.ncols + L.fl.nxtiles, kStageThreads / 32),
                         cdiv((long long)M.nruns * (M.maxnf + 1), kStageThreads),
                         cdiv((long long)L.al.nruns * L.al.maxn, kStageThreads), 1});
    launch_coop(k32_stage_pre, std::min(need, stage32_grid_limit(0)), L);
}

void launch_stage32_fct(const Stage32Launch &L) {
    const FctLaunch &F = L.fl;
    const int ti = F.tile_i > 0 ? F.tile_i : 8, per = ti >= 8 ? 1 : 8 / ti;
    int need = std::max({cdiv(F.ntiles, per), cdiv(F.nptiles, kStageThreads / 32),
                         cdiv(L.max_batch, kStageThreads), cdiv((long long)L.mx.nruns * L.mx.maxnf, kStageThreads), 1});
    launch_coop(k32_stage_fct, std::min(need, stage32_grid_limit(1)), L);
}

// ---------------------------------------------------------------- per-sub-step kernels
__global__ void k_ghost32(const PatchT<float> *patches, const GhostOp *ops, int n, int slot) {
    VX_PDL_WAIT();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) ghost_op(patches, ops, k, slot);
}
__global__ void k_iface32(const PatchT<float> *patches, const IfaceOp *ops, int n, int step) {
    VX_PDL_WAIT();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) iface_op(patches, ops, k, step);
}
__global__ void k_csync32(const PatchT<float> *patches, const CSyncOp *ops, int n) {
    VX_PDL_WAIT();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) csync_op(patches, ops, k);
}
__global__ void k_assemble32(AsmLaunch A) {
    VX_PDL_WAIT();
    const int run = blockIdx.y;
    if (run >= A.nruns) return;
    assemble_cell(A, run, blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void k_mx_rhs32(MaxwellLaunch L) {
    VX_PDL_WAIT();
    const int run = blockIdx.y;
    if (run >= L.nruns) return;
    mx_rhs_cell(L, run, blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void k_mx_update32(MaxwellLaunch L) {
    VX_PDL_WAIT();
    const int run = blockIdx.y;
    if (run >= L.nruns) return;
    mx_update_cell(L, run, blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void k_mx_asq32(MaxwellLaunch L) {
    VX_PDL_WAIT();
    const int run = blockIdx.y;
    if (run >= L.nruns) return;
    mx_asq_cell(L, run, blockIdx.x * blockDim.x + threadIdx.x);
}

void launch_ghost32(const void *patches, const GhostOp *ops, int n, int slot, cudaStream_t s) {
    if (n > 0) vx_launch(k_ghost32, (n + 127) / 128, 128, 0, s, (const PatchT<float> *)patches, ops, n, slot);
}
void launch_iface32(const void *patches, const IfaceOp *ops, int n, int step, cudaStream_t s) {
    if (n > 0) vx_launch(k_iface32, (n + 127) / 128, 128, 0, s, (const PatchT<float> *)patches, ops, n, step);
}
void launch_csync32(const void *patches, const CSyncOp *ops, int n, cudaStream_t s) {
    if (n > 0) vx_launch(k_csync32, (n + 127) / 128, 128, 0, s, (const PatchT<float> *)patches, ops, n);
}
void launch_assemble32(const AsmLaunch &A) {
    dim3 g((A.maxn + 255) / 256, A.nruns);
    vx_launch(k_assemble32, g, 256, 0, A.stream, A);
}
void launch_maxwell32(const MaxwellLaunch &L) {
    dim3 g((L.maxnf + 255) / 256, L.nruns);
    vx_launch(k_mx_rhs32, g, 256, 0, L.stream, L);
    vx_launch(k_mx_update32, g, 256, 0, L.stream, L);
    vx_launch(k_mx_asq32, g, 256, 0, L.stream, L);
}

}  // namespace vx
