// Serving loop: continuous batching of independent solves under an HBM budget (serve.cpp).
#pragma once
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "engine.hpp"

namespace vx {

class Server {
public:
    enum Status { kWaiting = 0, kBuilding, kLive, kDone, kCancelled, kFailed };
    struct Request {
        int64_t id = 0;
        LaserSlabParams params;
        int precision = kF64;
        int poisson = kPoissonLU;
        int regrid = 1;  // 1: the reference driver's regrid rule (veritas.cpp:146-151); 0: none
        int fast64 = 0;  // FP64 requests: the contracted FCT kernels
        int64_t steps = 0, done_steps = 0;
        int regrid_counter = 0;
        int regrids = 0;
        bool out = false;  // live, its run with a worker thread for a regrid
        double arrival = 0, admitted = -1, bound = -1, finish = -1, sim_time = 0;
        size_t estimate = 0, bytes = 0;
        long long cells = 0;
        Status status = kWaiting;
        std::string state_path, error;
        std::unique_ptr<Run> run;
    };

    Server(Engine &eng, size_t hbm_budget_bytes, int max_live);
    ~Server();
    // Queue a solve of `steps` RK steps that arrived at `arrival` (seconds on clock()).
    int64_t submit(const LaserSlabParams &p, int precision, int64_t steps, double arrival,
                   const std::string &state_path, int poisson = kPoissonLU, int regrid = 1, int fast64 = 0);
    // Advance every live solve one step; meanwhile bind the runs the workers finished,
    // admit what fits (its runs are built on the worker threads) and build the next
    // step's launch sets; then hand the solves whose counter says so to the workers for
    // their regrid and retire the finished, failed and cancelled ones.  Returns the live
    // count (solves out for a regrid included).
    int step(double now);
    // Withdraws a request that has not finished: a waiting one leaves the queue, one being
    // built is dropped when its build ends, a live one is retired now (no state written).
    void cancel(int64_t id);
    const Request &request(int64_t id) const;
    double clock() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
    }
    size_t used_bytes() const { return used_; }
    // Live solves, those out for a regrid included.
    int live() const { return (int)live_.size() + regridding_; }
    // Requests not yet live: waiting for memory, or admitted and being built.
    int waiting() const;
    static size_t estimate_bytes(const LaserSlabParams &p, int precision);
    // The regrid rule's time threshold [s]: the reference's driver regrids only once its
    // plasma is switched on (t > 3 laser periods in its demo, veritas.cpp:139-151); served
    // solves couple the plasma from t = 0, so the default is 0.  regrid_enabled = false
    // turns regridding off for every request.
    double regrid_after = 0;
    bool regrid_enabled = true;

private:
    // One job of a worker thread: an admitted request's run to build, or a live solve's
    // run to regrid (it sits out of the batch meanwhile).
    struct Build {
        int64_t id;
        bool regrid = false;
        LaserSlabParams params;
        int precision, poisson, fast64;
        std::unique_ptr<Run> run;
        std::string error;
    };
    static constexpr int kWorkers = 4;
    // Admits waiting requests in order while slots and budget allow (bound_meanwhile: runs
    // bound during the current step, not yet in live_).
    void admit(double now, int bound_meanwhile = 0);
    // Moves the runs the workers finished to `into` (live from then on).
    void bind_built(double now, std::vector<int64_t> &into);
    bool regrid_due(const Request &r, double t_before) const;
    void retire(Request &r, Status st, double now);
    void worker_loop(Engine *weng);
    Engine &eng;
    std::vector<std::unique_ptr<Engine>> worker_eng_;  // one per worker thread (own streams, same device)
    size_t budget_, used_ = 0;
    int max_live_;
    int64_t next_id_ = 1;
    std::map<int64_t, Request> reqs_;
    std::deque<int64_t> waiting_;
    std::vector<int64_t> live_;
    int building_ = 0, regridding_ = 0;
    std::vector<int64_t> finished_order_;
    std::chrono::steady_clock::time_point t0_ = std::chrono::steady_clock::now();
    double phase_s_[6] = {};  // VX_TRACE_SERVE: the loop's time per phase
    int hits_ = 0, misses_ = 0;
    std::vector<int64_t> predicted_;
    // worker threads: builds and regrids in (regrids first), finished runs out
    std::mutex mu_;
    std::condition_variable cv_, built_cv_;
    std::deque<Build> todo_;
    std::vector<Build> built_;
    bool stop_ = false;
    std::vector<std::thread> workers_;
};

}  // namespace vx
