// Device runtime: runs (one per SolverManager), their patches in HBM, and the launch
// sets that advance a group of runs together with one launch per sub-step.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "amr.hpp"
#include "poisson_lu.hpp"
#include "settings.hpp"
#include "vx_kernels.hpp"

namespace vx {

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
// A bounded device wait ran out (a persistent stage kernel's grid barrier).
struct TimeoutError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
void cuda_check(cudaError_t e, const char *what);
#define VX_CUDA(x) ::vx::cuda_check((x), #x)

// Owned device allocation.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    bool own = true;  // false: a view into storage another DevBuf owns
    DevBuf() = default;
    explicit DevBuf(size_t b);  // zero-filled
    struct Uninit {};
    DevBuf(size_t b, Uninit);   // contents undefined: for buffers the caller fills at once
    static DevBuf view(void *p, size_t b) {
        DevBuf d;
        d.p = p;
        d.bytes = b;
        d.own = false;
        return d;
    }
    ~DevBuf();
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), bytes(o.bytes), own(o.own) {
        o.p = nullptr;
        o.bytes = 0;
    }
    DevBuf &operator=(DevBuf &&o) noexcept;
    template <class T>
    T *as() const {
        return (T *)p;
    }
};

// Device copy of a host vector (at least one element's worth of storage).
template <class T>
DevBuf upload(const std::vector<T> &v, cudaStream_t s) {
    if (v.empty()) return DevBuf(sizeof(T));
    DevBuf b(v.size() * sizeof(T), DevBuf::Uninit{});
    VX_CUDA(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return b;
}

// Device tables packed into one allocation: host tables are staged back to back
// (256-byte aligned) and copied in one transfer, device-only regions reserved beside
// them; the DevBufs handed in become views of the allocation once allocate() has run.  A
// launch set's two dozen tables then cost one allocation and one copy instead of two
// dozen of each (and one free when the set goes).
class TablePack {
public:
    template <class T>
    void put(DevBuf &view, const std::vector<T> &v) {
        const size_t b = std::max<size_t>(v.size(), 1) * sizeof(T);
        const size_t off = host_.size();
        host_.resize(off + align(b), 0);  // an empty table: one zero element, as upload() gives
        if (!v.empty()) std::memcpy(host_.data() + off, v.data(), v.size() * sizeof(T));
        items_.push_back({&view, off, b, true});
    }
    // device-only region, contents undefined until a kernel writes it
    void reserve(DevBuf &view, size_t bytes) {
        bytes = std::max<size_t>(bytes, 1);
        items_.push_back({&view, dev_, bytes, false});
        dev_ += align(bytes);
    }
    // Bytes the tables take in one allocation.
    size_t bytes() const { return host_.size() + dev_; }
    // Points the views into `arena` (at least bytes() long); copy() then moves the staged
    // tables on `s` — when given page-locked staging (host and device addresses, at least
    // staged_bytes() long, not reused before `s` has run the copy), by a kernel reading it:
    // a transfer from pageable memory, or any copy-engine transfer, queues behind the
    // large uploads of other threads building runs.
    void place(const DevBuf &arena);
    size_t staged_bytes() const { return host_.size(); }
    void copy(cudaStream_t s, void *pinned_host = nullptr, void *pinned_dev = nullptr);

private:
    static size_t align(size_t b) { return (b + 255) / 256 * 256; }
    struct Item {
        DevBuf *view;
        size_t off, bytes;
        bool staged;
    };
    std::vector<char> host_;
    std::vector<Item> items_;
    size_t dev_ = 0;
    char *base_ = nullptr;
};

// Geometry of one Rectangle (Rectangle.hpp:20-23) plus its device storage.
struct Rect {
    int n_x = 0, n_p = 0, x_pos = 0, p_pos = 0, depth = 0;
    bool up = false, down = false, left = false, right = false;
    int species = 0;
    int pitch = 0;
    DevBuf slab;   // all per-patch planes
    DevBuf cols;   // chargeR, currentR
    DevBuf masks;  // nested, ifx, ifp (AMR only)
    // Device descriptor.  For FP32 runs the plane pointers address float planes: the
    // layout of PatchT<float> is identical (see the static_assert in engine.cpp), and the
    // host never dereferences them.
    PatchT<double> desc{};
    int esize = 8;  // bytes per element of the planes (8: FP64 path, 4: FP32 form)
    size_t plane_elems() const { return (size_t)(n_x + 4) * pitch; }
    size_t plane_bytes() const { return plane_elems() * esize; }
    // Connectivity (Rectangle.hpp:8-12): neighbour patch ids (flat index within the run)
    // or -1 for the domain boundary; "same level" flags; per-cell/face finer patch ids and
    // the nested / interface masks, indexed (i+2)*(n_p+4) + (j+2) as IndexNS.
    int id = -1;
    std::vector<int> xm, xp, pm, pp;
    std::vector<char> sxm, sxp, spm, spp;
    std::vector<int> finer, finer_x, finer_p;
    std::vector<uint8_t> nested, ifx, ifp;
    int ns(int i, int j) const { return (i + 2) * (n_p + 4) + (j + 2); }
};

class Engine;

// Geometry and boundary flags of one patch of a promoted hierarchy.
struct PatchGeom {
    int depth, x_pos, p_pos, n_x, n_p;
    bool up, down, left, right;
};

// One independent solve: the state owned by the reference's SolverManager
// (SolverManager.hpp:5-19): Settings, one mesh per species, the field solver.
class Run {
public:
    Run(Engine &eng, std::shared_ptr<Problem> prob, int precision = kF64);
    ~Run();
    Engine *eng;  // the engine whose stream runs this run's work (a serving loop builds on its own)
    // Hands the run to another engine of the same device: the old engine drops its cached
    // launch sets (call on the thread that drives the old engine, with its work done).
    void migrate(Engine &to);
    // Points the run at `to` when its engine has already dropped it (Engine::forget, called
    // on that engine's own thread): a thread that cannot touch the old engine takes it over.
    void adopt(Engine &to) { eng = &to; }
    std::unique_ptr<Settings> S;
    // rects[species][depth] -> patches of that level, in the reference's order.
    std::vector<std::vector<std::vector<std::unique_ptr<Rect>>>> rects;
    int n = 0, pre = 0, post = 0, nf = 0;
    double dx0 = 0;
    // fields
    DevBuf dBy, dBz, dEy, dEz, dAy, dAz, dasq, dphi, dcharge, dJ, dneut, defin, dex0, dasq32, defin32, dacell32;
    RunFields F{};
    PoissonLU lu;
    DevBuf dlu_perm, dlb_band, dlb_fptr, dlb_fcol, dlb_fval, dlb_slot, dlb_sload, dlb_take, dub_band, dub_diag, dub_rdiag, dub_rdlo, dub_fptr, dub_fcol,
        dub_fval;
    LUDev ludev{};
    std::vector<int> pipe_rfc;  // per row: first forward chunk reading it (empty: no pipelined solve)
    uint64_t layout_version = 0;
    int id = 0;
    int precision = kF64;            // kF64: plain path; kF32: precision form
    int poisson = kPoissonLU;        // Poisson solver (kF32 runs always use kPoissonScan)
    int fast64 = 0;                  // FP64 runs: 1 = the contracted FCT kernels (not the reference's rounding)
    std::vector<double> fnorm;       // per species: scale of the stored FP32 f (1 for FP64)
    // fast Poisson of the precision form (Woodbury columns and capacitance)
    std::vector<double> pf_Y;
    PoissonFastDev pfdev{};
    DevBuf dpf_Y;
    void build_poisson_fast();
    void rebase_neutralization(const std::vector<std::vector<double>> &f1_planes);
    size_t device_bytes() const;     // device memory held by this run

    // SolverManager-level operations (SolverManager.cpp:8-164).
    void init();                        // constructor path: hierarchy, f(t=0), fields, neutralisation
    double calculate_dt();              // cfl * EstimateCFLBound
    void advance(double dt);            // six RK stages
    void advance_fields(double dt);     // Maxwell-only stages

    // State exchange in the reference dump layout (see vx.h).
    void load_state(const std::string &path);
    void save_state(const std::string &path);

    long long cell_count() const;
    void allocate_rect(Rect &r);
    void upload_rect_desc(Rect &r, int run_index_in_set);
    void init_rect_distribution(Rect &r);  // Rectangle::InitializeDistribution on the host
    void alloc_fields();
    void upload_lu();
    void enforce_neutralization();
    // AMR: flat patch list (species -> depth -> patch), connectivity and op lists.
    std::vector<Rect *> flat;
    std::vector<GhostOp> ghost_ops;
    Batched ghost_b;
    std::vector<CSyncOp> csync_ops;
    Batched csync_b;
    std::vector<IfaceOp> iface_ops;
    Batched iface_b;
    DevBuf dghost_ops, dcsync_ops, diface_ops;  // the op lists on the device (set tables gather them)
    DevBuf drelc;                   // sub-cell interpolation weights per depth
    DevBuf drefc;                   // coarse-to-fine interpolation weights (refinement ratio)
    std::vector<int> relc_off;      // offset of depth d's weights in drelc
    DevBuf drelc32;                 // FP32 copy: per depth 3*rtb weights, then their 3 sums
    std::vector<int> relc32_off;
    bool multi_patch = false;
    void build_amr();               // connectivity + op lists + masks for the current layout
    void validate_ops() const;      // bounds of every op against its patches
    // Hierarchy construction / regridding (regrid.cpp)
    using BoxList = std::vector<std::pair<std::pair<int, int>, std::pair<int, int>>>;
    std::vector<std::vector<std::pair<int, int>>> flag_cells();
    std::vector<BoxList> hierarchy_of(int species) const;
    void regrid(bool init);         // Mesh::updateHierarchy for every species
    void promote(const std::vector<std::vector<BoxList>> &hier, bool init);
    void transfer_from(std::vector<std::vector<std::vector<std::unique_ptr<Rect>>>> &old);
    DevBuf flat_descs();
    void push_data(int slot);       // Mesh::PushData(slot) for this run
    void copy_slot(int from, int to);
    int64_t state_size() const;
    void step_host(const double *in, double *out, double dt);
    void state_to_host(double *out);
    // Diagnostics in the reference's text formats (output.cpp).
    void write_fields(const std::string &dir, unsigned mask, int digits, double t);
    void write_rectangles(const std::string &dir, double t);
    std::map<std::string, std::unique_ptr<std::ofstream>> out_streams;  // files kept open, by path
    std::ofstream &out_stream(const std::string &path, int digits);
    std::vector<double> slot_to_host(const Rect &r, int slot);
};

// Clustering of one species' hierarchy (Mesh::updateHierarchy without the promotion)
// and the geometry of the promoted patches; host only (regrid.cpp).
std::vector<Run::BoxList> update_hierarchy(const Settings &s, int sp, std::vector<Run::BoxList> H,
                                           const std::function<std::vector<std::pair<int, int>>(int)> &level_flags);
std::vector<PatchGeom> promote_geometry(const Settings &s, int sp, const std::vector<Run::BoxList> &H);
// Rectangle error weights (Rectangle.cpp:68-74) of a patch of depth `depth`.
void error_weights(const Settings &s, int depth, int sp, double *w);

// A set of runs advanced together: flattened descriptor and work tables.
struct LaunchSet {
    std::vector<Run *> runs;
    uint64_t key_version = 0;
    std::vector<PatchT<double>> hpatch;
    DevBuf dpatch, dtiles, dfields, dcolpatch, dcolidx, dlvl_ptr, dlvl_off, dlvl_patch, drun_n, drun_ns,
        drun_nl, dlu, dw, dfcoef, dparams, dcfl_spec, dcfl_out, dns, ddxinv;
    int ntiles = 0, ncols = 0, maxnp = 0, maxn = 0, maxnf = 0;
    std::vector<double> hparams;  // per run: 6 stages x (8 fct + 8 maxwell + 2 laser)
    std::vector<float> hparams32;
    DevBuf dparams32;
    std::vector<double> w, fcoef;
    // AMR op tables of all runs, batch by batch (global patch ids)
    DevBuf dghost, diface, dcsync;
    int precision = kF64;
    int tile_j = 32, tile_i = 8;  // FCT tile (p x x) = thread block of the sub-step kernels
    DevBuf dxtiles, dptiles;      // FP32: strip tiles of the fused face + flux kernels
    int nxtiles = 0, nptiles = 0;
    int poisson = kPoissonLU;
    int fast64 = 0;  // FP64 sets: contracted FCT kernels
    DevBuf dpf;  // per-run PoissonFastDev (scan Poisson sets)
    std::vector<int> ghost_ptr, iface_ptr, csync_ptr;
    DevBuf dghost_ptr, diface_ptr, dcsync_ptr;  // the batch offsets on the device (persistent form)
    int max_batch = 0;                          // largest op batch
    int launches_per_step = 0;                  // kernels of one recorded step
    // FP64 exact-solve sets of up to kPipeMaxRuns runs: tables of the pipelined moments +
    // solve launch (k64_moments_poisson)
    bool pipe = false;
    int pipe_nunits = 0, pipe_nitems = 0, pipe_ndone = 0, pipe_summers = 1;
    DevBuf dpipe_col0, dpipe_sig, dpipe_item0, dpipe_nwin, dpipe_c12, dpipe_items, dpipe_need, dpipe_runctr,
        dpipe_rungptr, dpipe_gptr, dpipe_grow, dpipe_scratch, dpipe_state;
    DevBuf arena, tile_arena;  // the storage of the tables above (TablePack), tiles rebuilt alone
    // built but not yet on the device (Engine::flush_set): the staged tables, the op
    // gathers, their segment lists
    std::unique_ptr<TablePack> pending_pack;
    std::vector<std::function<void()>> pending_gathers;
    DevBuf dsegs[3];
    cudaGraphExec_t graph = nullptr;
    ~LaunchSet();
};

// Launch descriptors of one set's step kernels (Engine::stage_launches).
struct StageLaunches {
    FctLaunch fl;
    MomLaunch ml;
    AsmLaunch al;
    PoissonLaunch pl;
    MaxwellLaunch mx;
};

// Phases of one RK stage for Engine::run_phases (the per-class entry points).
enum StagePhase : unsigned {
    kPhMoments = 1u,   // EMFieldSolver::AssembleRhoAndJ
    kPhPoisson = 2u,   // EMFieldSolver::UpdatePotential (+ E_x)
    kPhSub0 = 4u,      // Mesh::Advance sub-step 0 (fluxes, interface fluxes, low-order f)
    kPhSub1 = 8u,      // PushData(2), sub-step 1 (limiter), PushBoundaryC
    kPhSub2 = 16u,     // sub-step 2 (antidiffusive update), PushData(1)
    kPhSub3 = 32u,     // sub-step 3 (f0 = f1; stage 5 only)
    kPhMaxwell = 64u,  // EMFieldSolver::RGKStep
};

class Engine {
public:
    explicit Engine(int device);
    ~Engine();
    int device;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;       // Poisson solve beside the E-independent x-direction work
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_gamma = nullptr, ev_mx = nullptr;  // Maxwell stage beside the FCT chain
    std::vector<Run *> runs;
    bool use_graphs = true;
    uint64_t kernel_launches = 0;  // launches issued by this engine (graph replays count their nodes)

    void advance(const std::vector<Run *> &set, const std::vector<double> &dt);
    void advance_fields(const std::vector<Run *> &set, const std::vector<double> &dt);
    void fill_params(LaunchSet &L, const std::vector<Run *> &set, const std::vector<double> &dt);
    void run_phases(Run &run, int stage, double dt, unsigned phases);
    std::vector<double> calculate_dt(const std::vector<Run *> &set);
    void moments_only(const std::vector<Run *> &set);
    void refresh_efield(Run &run);
    // Mean device time per launch of each Vlasov kernel (see vx_run_profile_kernels).
    std::vector<double> profile_kernels(Run &run, int reps);
    void timer_begin();
    double timer_end();
    void flush_l2();
    double measure_fp64_peak();
    void measure_fp64_latency(double *mul_sub_cycles, double *shfl_cycles);
    void sync();
    void forget(Run *r);
    // Times the FCT sub-step kernels of the set for each candidate tile shape and keeps
    // the fastest for this precision (autotune.cpp).  Leaves the solution unchanged.
    std::pair<int, int> autotune(const std::vector<Run *> &set, int reps);
    // CUDA graph per step and programmatic dependent launch on or off; drops the
    // captured graphs (they hold the old launch attributes).
    void set_launch_mode(bool graphs, bool pdl);
    // FP32 sets: each RK stage as the persistent stage kernels (stage32.cu) instead of one
    // launch per sub-step; drops the captured graphs.
    void set_persistent(bool on);
    bool persistent = false;
    // Wait limit of the persistent kernels' grid barriers, and arrivals each barrier waits
    // for beyond the grid's (0; the failure test makes every wait run out with it).
    void set_persistent_limit(unsigned long long limit_ns, int phantom);
    unsigned long long persist_limit_ns = 2000000000ull;
    int persist_phantom = 0;
    // FP64 exact-solve sets: moments, assembly and solve in one launch whose solve follows
    // the moments as they finish (on by default; off: the three separate kernels, same bits).
    // Its waits use the persistent form's limit and phantom count.  Drops the captured graphs.
    void set_pipelined(bool on);
    bool pipelined = true;
    // Throws TimeoutError if a persistent kernel's barrier wait ran out since the last
    // check (called by sync(), once the stream is idle), clearing the record.
    void check_device_errors();
    // Drops every cached launch set but the listed ones (their tables and graphs hold
    // device memory; a serving loop keeps only the sets of its current step).
    void retain_sets(const std::vector<std::vector<Run *>> &keep);
    // Table storage of dropped launch sets, kept for the next sets (a serving loop builds
    // one almost every step, and cudaMalloc beside running kernels and other threads'
    // allocations costs milliseconds: a set's gathered op tables can take hundreds of MB);
    // at most arena_cache_limit bytes are kept.
    DevBuf take_arena(size_t bytes);
    size_t arena_cache_limit = (size_t)2 << 30;
    // Page-locked staging of at least `bytes` for the set tables' copy (grown as needed);
    // its device address in pinned_dev_.
    void *pinned_staging(size_t bytes);
    // Builds (or finds) the launch set of `set`, host work only: a serving loop prepares
    // the next step's sets while the current step runs.  The sets' table copies are
    // queued by flush_prepared() (or their first use).
    void prepare(const std::vector<Run *> &set);
    void flush_prepared();
    int tile_pref[2][2] = {{32, 8}, {128, 8}};  // [precision 64, 32] -> (tile_j, tile_i)

private:
    std::map<std::vector<Run *>, std::unique_ptr<LaunchSet>> sets_;
    std::multimap<size_t, DevBuf> arena_cache_;  // idle table storage by size
    void *pinned_ = nullptr, *pinned_dev_ = nullptr;
    size_t pinned_bytes_ = 0;
    cudaEvent_t ev_pinned_ = nullptr;  // after the last copy out of pinned_
    size_t arena_cache_bytes_ = 0;
    // Drops a launch set whose work has finished (the engine's stream synchronised): its
    // table storage goes to the cache.
    void drop_idle(std::unique_ptr<LaunchSet> &L);
    // defer: the set's table copy and gathers wait for flush_set / flush_prepared
    LaunchSet &get_set(const std::vector<Run *> &set, bool defer = false);
    void build_set(LaunchSet &L);
    void flush_set(LaunchSet &L);
    // pk: the set's table pack; none: the tiles are rebuilt alone (their own allocation)
    void build_tiles(LaunchSet &L, TablePack *pk = nullptr);
    void build_pipe_tables(LaunchSet &L, const std::vector<int> &colpatch, const std::vector<int> &colidx,
                           TablePack &pk);
    void record_step(LaunchSet &L);
    void capture_graph(LaunchSet &L);
    void record_step_persistent32(LaunchSet &L);
    StageLaunches stage_launches(LaunchSet &L);
    DevBuf gsync_;               // GridSyncState of the persistent kernels
    DevBuf stage_trace_;         // VX_TRACE_STAGE=1: clock trace of the persistent kernels of a step
    bool gsync_pending_ = false;  // persistent kernels ran since the last check
    DevBuf pipe_err_;             // the pipelined solve's wait record (PipeLaunch::err)
    bool pipe_pending_ = false;   // pipelined launches ran since the last check
    int prio_hi_ = 0;             // greatest stream priority of the device
    int num_sms_ = 1;
    PipeLaunch pipe_launch(LaunchSet &L, const StageLaunches &K);
    void record_pipe_stage(LaunchSet &L, StageLaunches &K, int s, int &launches);
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    DevBuf flush_;
};

}  // namespace vx
