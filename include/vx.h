/*
 * vx.h — C ABI of the GB300 Vlasov–Maxwell step (libvx_cuda.so).
 *
 * The reference (Veritas, C++14/OpenMP) has no plugin or FFI surface: its driver calls
 * C++ class methods.  Each entry point below replaces one of those methods for the
 * per-step path; the citation after each declaration names the reference interface it
 * stands in for (file:line in the Veritas source tree).
 *
 * Conventions
 *   - Every function returns 0 on success or a negative VX_ERR_* code; the message of
 *     the last failure on the calling thread is available from vx_last_error().  No
 *     function calls exit() (the reference exits on configuration errors,
 *     Settings.cpp:35-50).
 *   - A context owns one CUDA device and one stream; all device memory of its runs is
 *     owned by the context.  Host pointers passed in are borrowed for the call only.
 *   - Calls on one context must come from one thread at a time; different contexts are
 *     independent.
 */
#ifndef VX_H_
#define VX_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VX_OK 0
#define VX_ERR_INVALID -1   /* bad argument or configuration */
#define VX_ERR_CUDA -2      /* CUDA runtime error */
#define VX_ERR_STATE -3     /* operation not valid in the current state */
#define VX_ERR_IO -4        /* file read/write failure */
#define VX_ERR_NOMEM -5     /* device memory budget exceeded */
#define VX_ERR_TIMEOUT -6   /* bounded device wait expired */
#define VX_ERR_UNSUPPORTED -7

typedef struct vx_ctx vx_ctx;
typedef struct vx_run vx_run;

/* Built-in synthetic laser / plasma-slab problem: the hooks a Veritas user writes in
 * veritas.cpp (initialConditions :7, settingsOverride :36, InitialDistribution :107,
 * GetBY/GetBZ :80/:93, RefinementOverride :76).  Lengths in laser wavelengths, momenta
 * in m_e c, temperatures in keV. */
typedef struct vx_problem {
    double lambda;     /* laser wavelength [m] */
    double L;          /* domain length [lambda] */
    uint32_t nx, np, Lfinest, r;
    double pmax;       /* p in [-pmax, pmax] */
    double dens;       /* plateau density / n_c */
    double x1, x2, x3, x4; /* up-ramp [x1,x2], plateau [x2,x3], down-ramp [x3,x4] */
    double Te;         /* electron temperature [keV] */
    double p0;         /* drift momentum */
    double pert_amp, pert_k; /* density modulation amplitude and mode number */
    double a0, fwhm, delay;  /* laser amplitude, field-envelope FWHM and delay [periods] */
    double cfl, minEff, crit, sizeWeight;
    int32_t quadDepth;
    int32_t precision; /* 64: plain FP64 path; 32: FP32 precision form (f, fluxes and
                        * limiter in FP32 scaled by 1/peak of the initial f; moments
                        * accumulated and fields advanced in FP64; Poisson by prefix
                        * scans instead of the dense LU) */
    double bdens, bp0, bTe; /* beam population: density fraction of the slab, drift, temperature [keV] */
    int32_t poisson;   /* Poisson solver of precision-64 runs: 0 (default) the reference's
                        * dense LU in its rounding order; 1 the O(n) prefix-scan solve on a
                        * thread-block cluster (not the LU's rounding: about 4e-11 relative
                        * from it at n = 8192, growing as n^2 with the LU's own error).
                        * Precision-32 runs always use 1. */
    double mi, iTe, ipmax; /* mobile ions (second species) when mi > 0: mass mi m_e, charge
                            * +e, the electrons' density, temperature iTe [keV], momenta in
                            * [-ipmax, ipmax] m_i c */
    int32_t fast;      /* precision-64 runs: 0 (default) the FCT kernels in the reference's
                        * operations and order (bit-exact); 1 the same kernels with fused
                        * multiply-add and the WENO weights from one ratio (fewer FP64
                        * instructions; results differ from the exact form at rounding
                        * level, about 1e-15 relative in f per step).  Runs advanced
                        * together share it. */
} vx_problem;

/* Fills *p with the defaults of the 2048 x 256 single-level laser/slab case. */
void vx_problem_defaults(vx_problem *p);

/* ---------------------------------------------------------------- user problems
 * The reference's whole user surface is its problem file (veritas.cpp): the user fills
 * the Input / Particles / Output structs (initialConditions, veritas.cpp:7), edits the
 * Settings (Settings::settingsOverride, :36) and supplies InitialDistribution (:107),
 * GetBY / GetBZ (:80, :93, the laser at x = 0) and RefinementOverride (:76), then
 * recompiles.  Here the same hooks are C callbacks handed to vx_run_create_hooks: a
 * custom problem needs no rebuild of the library.  The structs mirror the reference's
 * (Settings.hpp:4-65) with fixed-size arrays for the per-species vectors. */
#define VX_MAX_SPECIES 8
#define VX_MAX_MISC 8

/* Input (Settings.hpp:4-11). */
typedef struct vx_input {
    double minEfficiency, dx, k, refinementCriteria, cfl, sizeWeight, preLength, postLength;
    uint32_t nx, r, Lfinest;
    double plasma_xl_bound, plasma_xr_bound;
    int32_t ntempEM;                 /* entries of tempEM in use */
    double tempEM[VX_MAX_MISC];
} vx_input;

/* Particles (Settings.hpp:13-20): entry s of each array belongs to species s. */
typedef struct vx_particles {
    int32_t nspecies;
    double mass[VX_MAX_SPECIES], charge[VX_MAX_SPECIES];
    uint32_t np[VX_MAX_SPECIES];
    double dp[VX_MAX_SPECIES], pmin[VX_MAX_SPECIES];
    int32_t nmisc[VX_MAX_SPECIES];  /* entries of misc[s] in use */
    double misc[VX_MAX_SPECIES][VX_MAX_MISC];
} vx_particles;

/* Output (Settings.hpp:22-33): nonzero = on. */
typedef struct vx_output {
    int32_t time, rectangleData, charge, energy, potential, EFieldLongitudinal, EFieldTransverse, BFieldTransverse,
        AFieldSquared;
    int32_t precision;
} vx_output;

/* Settings (Settings.hpp:35-65): what the hooks read, and what settings_override may
 * change (the fields the reference's Settings::settingsOverride may assign: dx, dp,
 * pmin, temp, tempEM, quadratureDepth, the grid scalars, ...).  temp[s] is the
 * reference's temp[s] (Particles::misc on entry), ntemp[s] its length. */
typedef struct vx_settings {
    double dx, time, minEfficiency, preLength, postLength, refinementCriteria, cfl, sizeWeight, plasma_xl_bound,
        plasma_xr_bound;
    int32_t nspecies;
    double m[VX_MAX_SPECIES], q[VX_MAX_SPECIES], m_inv[VX_MAX_SPECIES], dp[VX_MAX_SPECIES], fMax[VX_MAX_SPECIES],
        pmin[VX_MAX_SPECIES];
    int32_t ntemp[VX_MAX_SPECIES];
    double temp[VX_MAX_SPECIES][VX_MAX_MISC];
    int32_t ntempEM;
    double tempEM[VX_MAX_MISC];
    uint32_t x_size_finest, x_size, refinementRatio;
    int32_t maxDepth, quadratureDepth;
    uint32_t p_size[VX_MAX_SPECIES], p_size_finest[VX_MAX_SPECIES];
} vx_settings;

/* The problem hooks.  `user` is passed back to every callback.  The settings a callback
 * sees are those after settings_override, with the derived sizes, m_inv and fMax filled
 * in once the Settings are complete (the reference's DetermineMaximum calls
 * initial_distribution before that); `time` is not kept current (the laser hooks get
 * the time as an argument).  initial_distribution is called concurrently from several
 * host threads and must be thread-safe; the others from the calling thread.  Units are
 * SI, as in the reference. */
typedef struct vx_hooks {
    void *user;
    /* initialConditions (veritas.cpp:7): fill the structs, which arrive holding the
     * reference's defaults (Settings.hpp:4-33).  Required. */
    void (*initial_conditions)(void *user, vx_input *grid, vx_particles *particles, vx_output *output);
    /* Settings::settingsOverride (veritas.cpp:36).  Optional. */
    void (*settings_override)(void *user, vx_settings *s);
    /* Settings::InitialDistribution (veritas.cpp:107): f(x, p) of species at t = 0.  Required. */
    double (*initial_distribution)(void *user, const vx_settings *s, double x, double p, int species);
    /* Settings::GetBY / GetBZ (veritas.cpp:80, :93): the transverse B the laser imposes at
     * x (the solver asks for x = 0) and time t.  Optional (NULL: 0). */
    double (*get_by)(void *user, const vx_settings *s, double x, double t);
    double (*get_bz)(void *user, const vx_settings *s, double x, double t);
    /* Settings::RefinementOverride (veritas.cpp:76): nonzero refines the cell at cell
     * centre x and lower p face p whatever its error estimate.  Optional (NULL: never). */
    int (*refinement_override)(void *user, const vx_settings *s, double x, double p, int depth, int species);
} vx_hooks;

/* The reference's defaults of Input, Particles (one species) and Output (Settings.hpp:4-33). */
void vx_input_defaults(vx_input *grid, vx_particles *particles, vx_output *output);

/* SolverManager::SolverManager (SolverManager.cpp:8-26) for a problem given by hooks:
 * the Settings from initial_conditions and settings_override (Settings.cpp:5-54,
 * validation errors are VX_ERR_INVALID), the initial hierarchy from
 * initial_distribution's quadrature and the error estimate with refinement_override
 * (Mesh.cpp:8-50), the field solver and the neutralising charge.  precision 64 or 32 and
 * poisson as in vx_problem.  The hooks are kept for the life of the run (the laser hooks
 * are called every stage, refinement_override at every regrid). */
int vx_run_create_hooks(vx_ctx *ctx, const vx_hooks *hooks, int precision, int poisson, vx_run **out);
/* The run's Settings as the hooks see them (time current). */
int vx_run_settings(vx_run *run, vx_settings *out);

/* ---------------------------------------------------------------- per-class calls
 * The steps SolverManager::Advance (SolverManager.cpp:28-39) takes per RK stage, one entry
 * point each, for callers that drive the stages themselves.  Each launches on the
 * context stream without a CUDA graph; called in the reference's order —
 *   for stage in 0..5: vx_run_moments; vx_run_poisson; vx_run_vlasov_stage(stage, dt,
 *   VX_SUB_ALL); vx_run_update_time(stage, dt); vx_run_maxwell_stage(stage, dt)
 * — they give the same bits as vx_run_advance(dt). */
/* EMFieldSolver::AssembleRhoAndJ (EMSolver.cpp:104-122): moments of every patch
 * (Rectangle::CalculateRhoAndJ, Rectangle.cpp:157-282), interpolated to the finest grid
 * and summed over levels and species (Level.cpp:19-62). */
int vx_run_moments(vx_run *run);
/* EMFieldSolver::UpdatePotential (EMSolver.cpp:156-192): phi, Ex0 and E_x on the finest grid. */
int vx_run_poisson(vx_run *run);
/* Mesh::Advance(dt, stage) (Mesh.cpp:64-89) for every species: sub_mask selects its parts.
 * Level::FCTTimeStep sub-steps (Level.cpp:12-16 -> Rectangle::FCTTimeStep,
 * Rectangle.cpp:1255-1623) and the exchanges between them. */
#define VX_SUB_FLUX 0x1    /* sub-step 0: face values, fluxes (coarse/fine faces included), low-order f */
#define VX_SUB_LIMIT 0x2   /* PushData(2), sub-step 1 (limiter R and C), PushBoundaryC */
#define VX_SUB_UPDATE 0x4  /* sub-step 2 (antidiffusive update), PushData(1) */
#define VX_SUB_COPY 0x8    /* sub-step 3 (f0 = f1): at stage 5 only, as Mesh::Advance */
#define VX_SUB_ALL 0xf
int vx_run_vlasov_stage(vx_run *run, int stage, double dt, unsigned sub_mask);
/* Settings::UpdateTime (Settings.cpp:166-179). */
int vx_run_update_time(vx_run *run, int stage, double dt);
/* EMFieldSolver::RGKStep (EMSolver.cpp:194-202): the Maxwell stage with the laser of
 * get_by/get_bz at the run's current time, then a^2 on the faces. */
int vx_run_maxwell_stage(vx_run *run, int stage, double dt);
/* Mesh::getError(lvl, false) (Mesh.cpp:289-294 -> Rectangle::getError,
 * Rectangle.cpp:866-890): the flagged cells (i, j) of the patches of one species and
 * depth (0 = finest), in the reference's patch and loop order, as pairs in ij_out (up to
 * cap pairs); *count receives the total. */
int vx_run_flag(vx_run *run, int species, int depth, int32_t *ij_out, int cap, int *count);

const char *vx_last_error(void);

/* Context: one GPU + one stream. */
int vx_ctx_create(int device, vx_ctx **out);
/* Fails (VX_ERR_INVALID) while runs created on the context are still alive. */
int vx_ctx_destroy(vx_ctx *ctx);
/* Launch mode (no reference counterpart; both on by default): graphs != 0 replays each
 * step as one captured CUDA graph, pdl != 0 launches every kernel with programmatic
 * dependent launch (process-wide).  For debugging and timing; results do not depend on
 * it. */
int vx_ctx_set_launch_mode(vx_ctx *ctx, int graphs, int pdl);
/* Persistent stage form (no reference counterpart; off by default): on != 0 advances the
 * context's FP32 runs (alone or batched) with three launches per RK stage — one
 * cooperative kernel for the moments and rho/J assembly, the Poisson solve, and one
 * cooperative kernel for the whole FCT stage of every patch of every run with the
 * Maxwell stage beside it — instead of one launch per sub-step (FP64 runs are unaffected).
 * Same bits as the per-sub-step form.  The kernels' grid barriers wait a bounded time; a
 * wait that runs out is reported by the next call that synchronises the context
 * (vx_ctx_sync, vx_run_calculate_dt, state reads) as VX_ERR_TIMEOUT, after which that
 * step's results are not valid and the context stays usable. */
int vx_ctx_set_persistent(vx_ctx *ctx, int on);
/* Wait limit of those barriers in ns (default 2e9) and a count of arrivals each barrier
 * waits for beyond the launch's own blocks (default 0; any phantom > 0 makes every wait
 * run out — the failure path's test). */
int vx_ctx_set_persistent_limit(vx_ctx *ctx, uint64_t limit_ns, int phantom);
/* Pipelined moments and exact Poisson solve (no reference counterpart; on by default):
 * on != 0 runs, for FP64 runs with the exact solve advanced alone or in sets of up to four,
 * EMFieldSolver::AssembleRhoAndJ and UpdatePotential of each RK stage as one launch in
 * which the solve's forward sweep follows the moment columns as they are completed (the
 * columns go out in the order the sweep needs them) instead of starting after all of them.
 * Same bits as the separate kernels (on == 0).  Its waits are bounded by the limit and
 * phantom count of vx_ctx_set_persistent_limit; a wait that runs out is reported as
 * VX_ERR_TIMEOUT by the next call that synchronises the context. */
int vx_ctx_set_pipelined(vx_ctx *ctx, int on);
int vx_ctx_sync(vx_ctx *ctx);
/* Kernels launched by this context so far (graph replays count their nodes). */
int vx_ctx_kernel_launches(vx_ctx *ctx, uint64_t *out);

/* SolverManager::SolverManager (SolverManager.cpp:8-26): Settings from the problem hooks
 * (Settings.cpp:5-54), initial hierarchy and distribution (Mesh.cpp:8-50,
 * Rectangle.cpp:616-665), field solver set-up (EMSolver.cpp:6-89) and charge
 * neutralisation (EMSolver.cpp:621-629). */
int vx_run_create(vx_ctx *ctx, const vx_problem *prob, vx_run **out);
int vx_run_destroy(vx_run *run);

/* SolverManager::CalculateDt (SolverManager.cpp:162-164 -> EMSolver.cpp:631-664). */
int vx_run_calculate_dt(vx_run *run, double *dt);
/* SolverManager::Advance (SolverManager.cpp:28-39): one six-stage RK step of every
 * species and the fields.  Asynchronous on the context stream. */
int vx_run_advance(vx_run *run, double dt);
/* SolverManager::AdvanceFields (SolverManager.cpp:41-46): the six Maxwell stages only
 * (the reference driver's warm-up before the plasma is switched on). */
int vx_run_advance_fields(vx_run *run, double dt);
/* SolverManager::reGrid (SolverManager.cpp:48-57 -> Mesh::updateHierarchy,
 * Mesh.cpp:132-208): flag cells, re-cluster every level, move f to the new patches. */
int vx_run_regrid(vx_run *run);
/* Patches of the current hierarchy: writes up to cap records of 6 ints
 * (species, depth, x_pos, p_pos, n_x, n_p) in the reference's level order; *count
 * receives the total. */
int vx_run_layout(vx_run *run, int32_t *out, int cap, int *count);
/* Rectangle error weights (Rectangle.cpp:68-74) of a patch at `depth` and the
 * refinement criterion: a cell is flagged when
 *   w[0]|f(i+1,j)-f(i-1,j)| + w[1]|f(i,j+1)-f(i,j-1)| + w[2]|f(i+1,j)-2f(i,j)+f(i-1,j)|
 *   + w[3]|f(i,j+1)-2f(i,j)+f(i,j-1)| + w[4]|f(i,j)| > crit   (Rectangle.hpp:128-130).
 * Host only. */
int vx_error_weights(const vx_problem *prob, int species, int depth, double *w5, double *crit);
/* Mesh::updateHierarchy's clustering and Mesh::promoteHierarchyToMesh's patch geometry
 * (Mesh.cpp:132-208, 297-792, 803-826) on the host, without any device state.  patches:
 * npatches records (depth, x_pos, p_pos, n_x, n_p) of one species in level order;
 * flag_ptr[npatches + 1] / flag_ij: the flagged cells (i, j) of each patch in global
 * level coordinates, in Rectangle::getError order.  out receives up to cap records
 * (depth, x_pos, p_pos, n_x, n_p, up, down, left, right) of the new hierarchy; *count
 * the total. */
int vx_update_hierarchy(const vx_problem *prob, int species, const int32_t *patches, int npatches,
                        const int32_t *flag_ptr, const int32_t *flag_ij, int32_t *out, int cap, int *count);
/* Advance several runs of one context together, one launch per sub-step for all of
 * them (batched form).  dt[i] belongs to runs[i]. */
int vx_runs_advance(vx_run *const *runs, const double *dt, int nruns);
/* No reference counterpart.  Tile-shape autotuner: times the FCT sub-step kernels of the
 * runs' launch set for each candidate tile (p x x cells = one thread block) and keeps the
 * fastest for the set and for later sets of that precision.  Call between steps; the
 * solution is unchanged.  The chosen shape is returned in *tile_j, *tile_i. */
int vx_runs_autotune(vx_run *const *runs, int nruns, int *tile_j, int *tile_i);
/* CalculateDt of several runs of one context in one launch; dt[i] belongs to runs[i]. */
int vx_runs_calculate_dt(vx_run *const *runs, double *dt, int nruns);

/* Simulation time (Settings::time, Settings.cpp:166-179). */
int vx_run_time(vx_run *run, double *t);
/* Total phase-space cells of all patches of all species and levels. */
int vx_run_cell_count(vx_run *run, int64_t *cells);

/* Checkpoint / parity exchange in the binary layout the parity harness writes
 * ("VXST0001": time, dt, Ex0, field arrays with their 8 RK slots, then every patch's
 * 3-slot f block in the reference's Index3 order, Rectangle.hpp:96). */
int vx_run_load_state(vx_run *run, const char *path);
int vx_run_save_state(vx_run *run, const char *path);

/* Copy field arrays to host memory.  which: 0 By, 1 Bz, 2 Ey, 3 Ez, 4 Ay, 5 Az (slot 0,
 * n+pre+post values), 6 a_squared (n+1), 7 phi (n), 8 charge (n), 9 J (n), 10 E_x on the
 * finest grid (n).  *len receives the element count; out may be NULL to query it. */
int vx_run_get_field(vx_run *run, int which, double *out, int64_t *len);

/* ---- diagnostics in the reference's text formats --------------------------------- */

/* Files of SolverManager::fileOutput (SolverManager.cpp:102-159), one bit each for the
 * flags of Output (Settings.hpp:22-33); VX_OUT_ALL is Output's defaults (all on, with
 * precision 15). */
#define VX_OUT_CHARGE 0x01        /* charge.txt, one line per species (EMSolver.cpp:340-358) */
#define VX_OUT_ENERGY 0x02        /* dNdP_<species>.txt (EMSolver.cpp:361-378) */
#define VX_OUT_POTENTIAL 0x04     /* potential.txt (EMSolver.cpp:417-430) */
#define VX_OUT_EFIELD_LONG 0x08   /* EFieldLong.txt (EMSolver.cpp:381-394) */
#define VX_OUT_EFIELD_TRANS 0x10  /* EFieldTrans.txt (EMSolver.cpp:396-415) */
#define VX_OUT_BFIELD_TRANS 0x20  /* BFieldTrans.txt (EMSolver.cpp:432-451) */
#define VX_OUT_ASQUARED 0x40      /* ASquared.txt (EMSolver.cpp:453-466) */
#define VX_OUT_TIME 0x80          /* time.txt (EMSolver.cpp:468-477) */
#define VX_OUT_ALL 0xff

/* Replaces SolverManager::fileOutput(t) (SolverManager.cpp:102).  Appends one record to
 * each selected file under dir (the reference writes under "output/"); a run creates its
 * files on its first call and appends afterwards, as the reference's streams do.  digits
 * is Output::precision (std::setprecision of the scientific values); t is written to
 * time.txt.  Values are formatted as the reference does, so an FP64 run's files compare
 * line by line with the reference's. */
int vx_run_write_fields(vx_run *run, const char *dir, uint32_t mask, int digits, double t);
/* Replaces SolverManager::OutputRectangles(t) / Mesh::outputRectangleData
 * (SolverManager.cpp:64-70, Mesh.cpp:877-902): writes
 * dir/rectangleData_p<species>_l<level>_t<t in scientific>.txt for every non-empty level
 * (the reference's dir is "output/rectangleData"). */
int vx_run_write_rectangles(vx_run *run, const char *dir, double t);

/* ---- measurement and host-buffer entry points ------------------------------------ */

/* Device time between two points on the context stream (CUDA events). */
int vx_ctx_timer_begin(vx_ctx *ctx);
int vx_ctx_timer_end(vx_ctx *ctx, double *ms);

/* Time the run's Vlasov kernels in isolation: reps back-to-back launches per kernel on
 * the context stream (after one untimed launch).  out_ms[k] receives the mean launch
 * time of kernel k in the order gamma, faces, flux, ds_f2, limR, limC, update,
 * moments (log table + ordered sums), assemble, poisson, maxwell, ghost, iface, csync
 * (all batches of each kind), moments_poisson (the pipelined moments + assembly + exact
 * solve launch; 0 where the run does not use it); *count is set to the number of entries
 * written (<= cap).  Each timed kernel is idempotent, so the run's state is unchanged. */
int vx_run_profile_kernels(vx_run *run, int reps, double *out_ms, int cap, int *count);

/* Overwrite a device buffer larger than the L2 cache on the context stream, so the next
 * timed region starts with a cold L2. */
int vx_ctx_flush_l2(vx_ctx *ctx);

/* Measured FP64 FMA throughput of this GPU in GFLOP/s (2 flops per FMA): a register-
 * resident DFMA chain kernel timed with CUDA events on the context stream. */
int vx_ctx_measure_fp64_peak(vx_ctx *ctx, double *gflops);
/* Dependent-chain latency of one lane in SM clock cycles: a multiply followed by a
 * subtract (the triangular solves' step) and the extra cost of a 64-bit shuffle in the
 * chain.  With them the exact Poisson solve's latency bound is stated. */
int vx_ctx_measure_fp64_latency(vx_ctx *ctx, double *mul_sub_cycles, double *shfl_cycles);

/* Page-locked host memory for host-buffer calls. */
int vx_host_alloc(size_t bytes, void **out);
int vx_host_free(void *p);

/* Packed host image of a run's state at a step boundary: every patch's f (slot 0,
 * padded (n_x+4) x pitch block, patch order species -> level -> patch), then the six
 * transverse field arrays (slot 0, n+pre+post each), a_squared (n+1), phi (n) and Ex0.  *len
 * receives the element count. */
int vx_run_state_size(vx_run *run, int64_t *len);
/* Copy the run's current state into a packed host image (D2H only). */
int vx_run_state_to_host(vx_run *run, double *state_out);
/* End-to-end step with host buffers (Veritas's driver loop calling
 * SolverManager::Advance on state that lives in host memory): copy state_in to the
 * device, run one RK step with dt, copy the new state to state_out. */
int vx_run_step_host(vx_run *run, const double *state_in, double *state_out, double dt);

/* ---------------------------------------------------------------- no-allocation CFL bound
 * No counterpart in the reference.  For callers that must not allocate device memory
 * (a time-step controller beside solves whose memory is committed up front, or one that
 * must not cause the synchronisation cudaMalloc / cudaFree may imply): the bound of
 * vx_run_calculate_dt (EMFieldSolver::EstimateCFLBound) from device field arrays the
 * caller owns — Ay, Az, By, Bz (their first n entries, slot 0) and E_x (n) — with the
 * species' charge q, mass m and finest-level dp0 given on the host.  Its scratch is a
 * fixed device array of VX_CFL_NOALLOC_MAX_CELLS / 256 doubles, looked up on the first
 * call on each device (make that first call before any stream capture, and do not use the
 * entry point on a device after cudaDeviceReset); larger n is rejected with
 * VX_ERR_INVALID, as are non-positive or non-finite dp0 and m.  Calls that overlap on the
 * GPU share the scratch and race.
 * `stream` is a cudaStream_t (NULL: the default stream); the call waits for its result. */
#define VX_CFL_NOALLOC_MAX_CELLS (1 << 20)
int vx_cfl_bound_noalloc(const double *Ay, const double *Az, const double *By, const double *Bz, const double *Ex,
                         int n, const double *q, const double *m, const double *dp0, int nspecies, double dx0,
                         double cfl, void *stream, double *dt);

/* ---------------------------------------------------------------- serving loop
 * No reference counterpart (the reference runs one solve per process): continuous
 * batching of independent solves on one context under a device-memory budget.
 * submit() queues a solve of `steps` RK steps (arrival on the server's clock, seconds;
 * a request larger than the whole budget is refused with VX_ERR_INVALID); step() binds
 * the runs its worker threads have finished, admits in arrival order the waiting solves
 * that fit in the budget (their runs are built on those threads while the batch keeps
 * stepping), advances every live solve one step in one batched launch set, regrids by
 * the reference driver's rule (on a worker thread, the solve out of the batch until its
 * new hierarchy is in place; it stays VX_REQ_LIVE), and retires the finished ones (writing their final state
 * to state_path when one was given) and the failed ones: a solve whose CFL bound or E_x0
 * is not finite after a step (something in it went non-finite) is retired alone with
 * VX_REQ_FAILED. */
typedef struct vx_server vx_server;
#define VX_REQ_WAITING 0    /* queued for device memory */
#define VX_REQ_BUILDING 1   /* admitted; its run is being built on a server worker thread */
#define VX_REQ_LIVE 2       /* stepping with the batch */
#define VX_REQ_DONE 3       /* all steps taken (state written if asked) */
#define VX_REQ_CANCELLED 4  /* withdrawn by vx_server_cancel */
#define VX_REQ_FAILED 5     /* build failed, or its fields went non-finite (error says which) */
typedef struct vx_request_result {
    int32_t finished;                 /* 1 once the request is over (done, cancelled or failed) */
    int64_t steps_done;
    double arrival, admitted, finish; /* server clock, seconds; -1 until reached */
    double sim_time;                  /* simulated time at the end of the solve */
    int64_t cells;                    /* phase-space cells of the final hierarchy */
    uint64_t device_bytes;            /* device memory the solve held */
    int32_t status;                   /* VX_REQ_* */
    int32_t regrids;                  /* regrids taken during the solve */
    double bound;                     /* server clock when its built run joined the batch; -1 until then */
    char error[192];                  /* why it failed (empty otherwise) */
} vx_request_result;
int vx_server_create(vx_ctx *ctx, uint64_t hbm_budget_bytes, int max_live, vx_server **out);
int vx_server_destroy(vx_server *s);
int vx_server_clock(vx_server *s, double *now);
int vx_server_submit(vx_server *s, const vx_problem *p, int64_t steps, double arrival, const char *state_path,
                     int64_t *id);
int vx_server_step(vx_server *s, int *live, int *waiting);
int vx_server_result(vx_server *s, int64_t id, vx_request_result *out);
/* Withdraws a request that is not over: a waiting one leaves the queue, one being built is
 * dropped when its build ends, a live one is retired at once (no state written). */
int vx_server_cancel(vx_server *s, int64_t id);
/* Regridding of served solves: enable != 0 applies the reference driver's rule
 * (veritas.cpp:146-151: SolverManager::reGrid when more than 20 steps have passed since
 * the last one, once the time before the step exceeds after_s seconds; the reference's
 * demo switches its plasma on at 3 laser periods, served solves at t = 0, so the default
 * is 0).  On by default. */
int vx_server_set_regrid(vx_server *s, int enable, double after_s);

#ifdef __cplusplus
}
#endif
#endif /* VX_H_ */
