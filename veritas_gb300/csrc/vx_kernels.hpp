// Kernel launch interfaces shared by the CUDA translation units and the host runtime.
#pragma once
#include <cuda_runtime.h>

#include <utility>

#include "vx_common.hpp"

namespace vx {

// Programmatic dependent launch.  Every kernel is launched with programmatic stream
// serialisation, so the next kernel on a stream is scheduled while the current one
// drains (the launch latency between the many short kernels of a stage overlaps the
// previous kernel's tail instead of following it).  Correctness rests on every kernel
// beginning with VX_PDL_WAIT: griddepcontrol.wait returns once the preceding grid has
// completed and its memory operations are visible (and at once for a kernel launched
// without the attribute), before the kernel reads or writes anything.
#define VX_PDL_WAIT() asm volatile("griddepcontrol.wait;" ::: "memory")
extern bool g_launch_pdl;  // cleared by vx_ctx_set_launch_mode (debugging, timing)
template <typename... KP, typename... A>
inline void vx_launch(void (*kernel)(KP...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream, A &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = g_launch_pdl ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);  // errors surface through cudaGetLastError
}
// Without the attribute: for the launch-set table kernels, queued from the host behind a
// running step's graph (nothing to overlap with there).
template <typename... KP, typename... A>
inline void vx_launch_plain(void (*kernel)(KP...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                            A &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

// One 32(p) x 8(x) tile of a patch's padded block; (i0, j0) is its lower corner in
// reference indices (>= -2).
struct TileRef {
    int patch, i0, j0;
};

// Per-run, per-stage parameter block in device memory (doubles):
//   [0..5]  FCT RK weights a_{s,k} * dt (Rectangle.cpp:1396-1517), [6] their sum,
//   [8..13] Maxwell stage weights (EMSolver.cpp:204-338),
//   [16] GetBY(0, t_s), [17] GetBZ(0, t_s) with t_s the time after UpdateTime(s).
constexpr int kParamStride = 18;
VX_HD inline int param_base(int run, int step) { return (run * 6 + step) * kParamStride; }

enum FctSub : int {
    kSubGamma = 0,
    kSubFaces,
    kSubFlux,
    kSubDsF2,
    kSubLimR,
    kSubLimC,
    kSubUpdate,
    kSubCopy10,
    // FP32 form only: gamma + x faces + x fluxes, and p faces + p fluxes, each fused
    kSubXFlux,
    kSubPFlux,
};

struct FctLaunch {
    const void *patches;  // device array of PatchT<T>
    const TileRef *tiles;
    int ntiles;
    const RunFields *fields;  // device array, one per run
    const double *params;     // per-run stage parameter blocks
    const float *params32;    // the same blocks in FP32 (FP32 form)
    int step;
    int use_f0;
    int part;  // faces / flux: 1 x faces only, 2 p faces only, 0 both
    int tile_j, tile_i;  // thread block = one tile of tile_j (p) x tile_i (x) cells
    // FP32 fused face + flux kernels: one warp per strip tile
    const TileRef *xtiles, *ptiles;
    int nxtiles, nptiles;
    cudaStream_t stream;
};
constexpr int kStripRows = 16;  // rows per strip tile of the fused FP32 face + flux kernels
constexpr int kXCols = 30;      // output columns per x strip (32 lanes hold j0-1 .. j0+30)

void launch_fct64_substep(const FctLaunch &L, int sub);
// The FP64 kernels compiled with contraction and the 3-division WENO weights (fast form).
void launch_fct64_substep_fast(const FctLaunch &L, int sub);
void launch_fct32_substep(const FctLaunch &L, int sub);

// ---------------------------------------------------------------- moments
struct MomLaunch {
    const void *patches;
    const int *colpatch;  // per moment column: patch index
    const int *colidx;    // per moment column: local column index c = i*rtb + k
    int ncols;
    int maxnp;            // largest n_p over the patches
    const RunFields *fields;
    int nruns, maxnf;     // FP32: the per-cell A^2 copy covers every run's field grid
    int acell = 1;        // FP32: refresh the per-cell A^2 copy first (else the Maxwell stage made it)
    int asq32 = 1;        // FP32: the moments kernel also makes the FP32 copy of a^2
    int fast = 0;         // FP64: the fast form's moments (fused multiply-adds, Newton reciprocal)
    cudaStream_t stream;
};
constexpr int kMomCols = 15;  // FP64 moment columns per block (padded per patch), plus a summing warp
constexpr int kMomWindow = 29;  // p cells per window of the FP64 moments (a warp's lanes 1..29)
void launch_moments64(const MomLaunch &M);
void launch_moments32(const MomLaunch &M);

// Assembly of rho and J on the finest grid (EMSolver::AssembleRhoAndJ).
struct AsmLaunch {
    const void *patches;
    const int *lvl_ptr;    // per run, (ns*nl + 1) absolute offsets into lvl_patch
    const int *lvl_off;    // per run: offset of its lvl_ptr block
    const int *lvl_patch;  // patch indices level by level, in each level's patch order
    const int *run_n;      // per run: n
    const int *run_ns;     // per run: species count
    const int *run_nl;     // per run: level count
    int nruns, maxn;
    int pairs;             // FP32 sets: a column holds its unscaled sum as an FP32 pair
    RunFields *fields;
    cudaStream_t stream;
};
void launch_assemble(const AsmLaunch &A);

// Poisson solve with precomputed sparse LU factors (EMSolver::UpdatePotential).
// One triangular factor in band form (see k_poisson): band[4*i + d - 1] is the
// coefficient of column i-d (L) or i+d (U), exact zero where the factor has none; the
// far entries of row i are fcol/fval[fptr[i] .. fptr[i+1]) in summation order.
struct BandFactor {
    const double *band;
    const double *diag;   // U: u_ii
    const double *rdiag;  // U: RN(1/u_ii)
    const double *rdiag_lo;  // U: 1/u_ii - RN(1/u_ii)
    const int *fptr, *fcol;
    const double *fval;
    int nslots;                // L: accumulator lanes in use (-1: far terms on lane 3)
    const double *slot_coef;   // L: [slot][step] coefficient of column step-1
    const int *slot_load;      // L: [slot][step] row whose right-hand side the slot takes up, or -1
    const int *take;           // L: [step] slot finishing row step+4, or -1
    int far_pre_col;           // U: see PoissonLU::Band (-1: none)
};

struct LUDev {
    int n;
    const int *perm;  // row interchanges composed into one gather b'[k] = b[perm[k]]
    BandFactor L, U;
};
struct PoissonLaunch {
    const LUDev *lu;      // per run
    RunFields *fields;    // per run (device array)
    const double *w;      // per run: dx0^2
    const double *fcoef;  // per run: 1/(12 dx0)
    int nruns;
    int maxn;
    int x_in_smem;  // set by launch_poisson
    unsigned long long *trace;  // optional: clock64 at the solve's phase and chunk ends (run 0)
    cudaStream_t stream;
};
void launch_poisson(const PoissonLaunch &L);
constexpr int kPoisRowsHost = 256;  // rows per chunk of k_poisson (fields64.cu kPoisRows)

// Moments, assembly and exact Poisson solve of an FP64 set in one launch
// (k64_moments_poisson): blocks 0 .. nruns-1 solve, each following its run's moments as
// they are completed; the other blocks are persistent workers.  Column warps (two groups
// of 15 per worker block) take items — one p window of one moment unit's 15 columns (one
// pair of sub-columns) — by ticket in the order the forward sweeps first need the units'
// columns, and write each cell's charge and current contributions to `scratch`; the warp
// that completes a unit's last item queues the unit.  Summing warps (four per summing
// block, one per sub-partition) take queued units in order, add their contributions in
// ascending p (the reference's order) and add one to the done counter of the chunk that
// needs the unit first.  The solve waits (bounded) for a chunk's counter before it
// assembles rho and J at the x positions whose right-hand sides the chunk reads first.
constexpr int kPipeErr = 0, kPipeTicket = 32, kPipeLeave = 64, kPipeQHead = 96, kPipeQTail = 128,
              kPipeDone = 160;  // words of the state (each on its own 128-byte line)
constexpr int kPipeMaxRuns = 4;  // sets of more runs keep separate launches (each solve holds an SM)
constexpr int kPipeItemDoubles = 2 * 32 * 30;  // per item: [cc, cj][lane t][column w][sub-column q]
constexpr size_t kPipeMaxScratch = (size_t)2 << 30;  // larger sets keep separate launches
struct PipeLaunch {
    MomLaunch M;             // moment columns (padded per patch into units of kMomCols)
    AsmLaunch A;             // assembly tables
    PoissonLaunch P;         // solve (x_in_smem set by the launcher)
    const int *unit_col0;    // per unit: its first column in M's column list
    const int *unit_sig;     // per unit: done counter it adds to
    const int *unit_item0;   // per unit: its first item (a unit's items are consecutive tickets)
    const int *unit_nwin;    // per unit: p windows per sub-column pair
    const double2 *unit_c12; // per unit: (1 / m) / c and its reciprocal, as the moments form them
    int nunits;
    const int *item_unit;    // per item: its unit
    int nitems;
    double *scratch;         // kPipeItemDoubles per item
    const int *need;         // per done counter: units that add to it
    int ndone;               // done counters; the units' item counters follow them
    const int *run_ctr;      // per run: its chunk-0 done counter
    const int *run_gptr;     // per run: offset of its (nchunks + 1) row pointers in gptr
    const int *gptr;         // rows first read by each forward chunk: grow[gptr[c] .. gptr[c+1])
    const int *grow;
    unsigned *state;         // kPipe* words; from kPipeDone: done counters, item counters, queue (zeroed by the last block out)
    int *err;                // 0, or 1 + the done counter whose wait ran out (or 1 + ndone: a summing warp's wait)
    unsigned long long limit_ns;
    int phantom;             // units each wait expects beyond the real ones (> 0: every wait runs out)
    int priority;            // launch priority (the moments go ahead of the face kernels beside them)
    int summers;             // summing blocks
    int workers;             // column-warp blocks
    // Optional globaltimer trace (ns) of run 0: [0] the solve's start, [1 + c] chunk c's rows
    // ready, [1 + trace_nch + k] the last unit of done counter k summed; the solve's own
    // chunk ends go to P.trace.
    unsigned long long *trace;
    int trace_nch;
    cudaStream_t stream;
};
void launch_moments_poisson64(const PipeLaunch &K);

// O(n) Poisson solve by prefix scans, one thread-block cluster per run (poisson_scan.cu).
// Y holds the m x 3 Woodbury columns (row-major), K the 3x3 capacitance factor.
constexpr int kPsMaxThreads = 512, kPsCluster = 8;
constexpr int kPsMaxSeg = 48;                                              // elements per thread
constexpr int kPsMaxUnknowns = kPsMaxThreads * kPsCluster * kPsMaxSeg;     // n - 1 <= this
struct PoissonFastDev {
    const double *Y;
    double K[9];
    double rho, c_inv, w1, w2;
};
struct PoissonFastLaunch {
    const PoissonFastDev *pf;  // per run
    RunFields *fields;         // per run (device array)
    const double *w;           // per run: dx0^2
    const double *fcoef;       // per run: 1/(12 dx0)
    int nruns;
    int maxn;                  // largest n of the runs
    int f32;                   // also write the FP32 copy of E_x (precision-32 sets)
    cudaStream_t stream;
};
void launch_poisson_fast(const PoissonFastLaunch &L);
size_t poisson_scan_smem(int maxn);  // dynamic shared memory of one block
// E_x from phi; f32 != 0 also writes its FP32 copy (precision-32 sets).
void launch_efield(RunFields *fields, const double *fcoef, int nruns, int maxn, int f32, cudaStream_t s);

// Maxwell RK stage + face interpolation of A (EMSolver::RGKStep).
struct MaxwellLaunch {
    RunFields *fields;  // device array
    int nruns, maxnf;
    int step;
    const double *params;  // per-run stage parameter blocks
    const double *dxinv;   // per run: 1/dx0
    int f32;               // precision-32 sets: also the FP32 per-cell A^2 (k_mx_update)
    int asq32_out = 0;     // the face a^2 step also writes the FP32 copy of a^2 (persistent form:
                           // nothing reads that copy between this step and the next stage)
    cudaStream_t stream;
};
void launch_maxwell(const MaxwellLaunch &L);

// CFL bound (EMSolver::EstimateCFLBound), result per run into out[run].
struct CflLaunch {
    const RunFields *fields;
    int nruns, maxn;
    const double *spec;   // per run: [ns][3] = |q|, m, dps ; followed by dpsMax
    const int *run_ns;
    double *out;
    cudaStream_t stream;
};
void launch_cfl(const CflLaunch &L);

// Interior of a fresh (zeroed) FP32 patch from the separable quadrature's 1-D sums.
void launch_fill_separable(float *f0, float *f1, int pitch, int nx, int np, const double *dx_sum,
                           const double *dp_sum, double inv, double fn, cudaStream_t s);
// FP64 initial cell averages of a product-form problem (see k64_quadrature): X[t][i*nvals
// + k], Pf[t][j*nvals + l] the factors at the sample points, C[t] the divisors.
void launch_quadrature64(double *f0, double *f1, int pitch, int nx, int np, int nvals, int terms, const double *X,
                         const double *Pf, const double *C, double scale, cudaStream_t s);
// FP64 FMA throughput probe: blocks x threads threads, iters x 8 independent DFMA each.
void launch_fp64_peak(double *out, int blocks, int threads, int iters, cudaStream_t s);
// One warp: cycles of iters dependent (multiply, subtract) steps, then with a shuffle each.
void launch_fp64_latency(long long *cyc, double *val, int iters, cudaStream_t s);

// AMR op batches (amr.hpp, amr64.cu)
struct GhostOp;
struct IfaceOp;
struct CSyncOp;
// `prec` selects the patch storage type (kF64 or kF32) of the descriptor array.
void launch_ghost(const void *patches, const GhostOp *ops, int n, int slot, int prec, cudaStream_t s);
void launch_iface(const void *patches, const IfaceOp *ops, int n, int step, int prec, cudaStream_t s);
// Launch-set op tables gathered on the device: segment s copies count ops from src to
// dst + dst_off and adds base to their patch ids (the run's first patch in the set).
struct OpSegment {
    const void *src;
    long long dst_off;
    int count, base;
};
void merge_ghost_ops(const OpSegment *segs, int nseg, GhostOp *dst, cudaStream_t s);
// bytes (a multiple of 16) from page-locked host memory, given by its device address, to
// device memory, copied by a kernel
void copy_from_host(const void *src_dev, void *dst, size_t bytes, cudaStream_t s);
void merge_iface_ops(const OpSegment *segs, int nseg, IfaceOp *dst, cudaStream_t s);
void merge_csync_ops(const OpSegment *segs, int nseg, CSyncOp *dst, cudaStream_t s);
void launch_csync(const void *patches, const CSyncOp *ops, int n, int prec, cudaStream_t s);
struct FlagPatch;
struct XferOp;
void launch_flags(const void *patches, const FlagPatch *fp, int n, uint8_t *out, int prec, cudaStream_t s);
void launch_xfer(const void *patches, const XferOp *ops, int n, uint8_t *mask, int prec, cudaStream_t s);

// dst[i] = -src[i]
void launch_negate(double *dst, const double *src, int n, cudaStream_t s);

// ---------------------------------------------------------------- FP32 launch sets (stage32.cu)
// The op batches, assembly and Maxwell stage of FP32 launch sets, as kernels over the same
// bodies as the persistent stage kernels below (one compilation, so the per-sub-step and
// the persistent forms give the same bits).
void launch_ghost32(const void *patches, const GhostOp *ops, int n, int slot, cudaStream_t s);
void launch_iface32(const void *patches, const IfaceOp *ops, int n, int step, cudaStream_t s);
void launch_csync32(const void *patches, const CSyncOp *ops, int n, cudaStream_t s);
void launch_assemble32(const AsmLaunch &A);
void launch_maxwell32(const MaxwellLaunch &L);

// Persistent form of an FP32 launch set's RK stage: two cooperative launches per stage
// around the Poisson solve, each running its phases over every patch of every run, the
// phases separated by grid-wide barriers.  A barrier waits at most limit_ns (and a fixed
// number of polls); a wait that runs out records 1 + its barrier index in err, and every
// later barrier of that and following launches passes without waiting until the host has
// read and cleared it, so a lost block can only cost time, never hang the stream.
struct GridSyncState {
    unsigned arrive;      // barrier arrivals of the running launch (the last block out resets it)
    unsigned pad0[31];
    unsigned released;    // barriers of the running launch whose last arrival has come
    unsigned pad1[31];    // (its own 128-byte line: the waiting blocks poll it, the arrivals add elsewhere)
    unsigned leave;       // blocks that finished the running launch
    int err;              // 0, or the index (from 1) of the first barrier whose wait ran out
    unsigned pad2[30];
    unsigned next;        // work counter of the running phase (reset by each barrier's release)
    unsigned pad3[31];
};
struct Stage32Launch {
    FctLaunch fl;      // patches, tile and strip lists, fields, FP32 stage weights
    MomLaunch ml;      // moments (acell: refresh the per-cell A^2 copy first)
    AsmLaunch al;      // assembly of rho and J
    MaxwellLaunch mx;  // Maxwell stage
    const GhostOp *ghost;  // op tables and their batch offsets (device arrays)
    const int *ghost_ptr;
    int nghost_b;
    const IfaceOp *iface;
    const int *iface_ptr;
    int niface_b;
    const CSyncOp *csync;
    const int *csync_ptr;
    int ncsync_b;
    int max_batch;     // largest op batch (grid sizing)
    int step;          // RK stage 0..5
    GridSyncState *sync;
    unsigned long long limit_ns;
    int phantom;       // arrivals each barrier waits for beyond the grid's (0; > 0 makes every wait run out)
    // Optional clock trace (kStageTraceSlots per launch, ns): [0] the launch's start on
    // block 0, [2k - 1] the last arrival at barrier k, [2k] block 0 leaving it.
    unsigned long long *trace;
    cudaStream_t stream;
};
constexpr int kStageTraceSlots = 128;
// [per-cell A^2 and a^2 copies] | moments + x fluxes | assembly: the x fluxes need neither
// E_x nor rho, so they run beside the moments, before the Poisson solve that separates the
// two launches; the FP32 a^2 copy they read comes from the previous stage's Maxwell step
// (MaxwellLaunch::asq32_out), or at stage 0 from the copy phase
void launch_stage32_pre(const Stage32Launch &L);
// p fluxes + Maxwell right-hand side | interface flux batches | ds/f2 + Maxwell update |
// ghost batches (f2) | limiter R + face a^2 | limiter C | C exchange batches | update |
// ghost batches (f1) | [f0 = f1]
void launch_stage32_fct(const Stage32Launch &L);
// Blocks of each persistent kernel one launch may use (co-resident on every SM).
int stage32_grid_limit(int which_fct);

}  // namespace vx
