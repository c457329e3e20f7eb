// Serving loop: continuous batching of independent solves under an HBM budget (serve.cpp).
#pragma once
#include <chrono>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "engine.hpp"

namespace vx {

class Server {
public:
    struct Request {
        int64_t id = 0;
        LaserSlabParams params;
        int precision = kF64;
        int poisson = kPoissonLU;
        int64_t steps = 0, done_steps = 0;
        double arrival = 0, admitted = -1, finish = -1, sim_time = 0;
        size_t estimate = 0, bytes = 0;
        long long cells = 0;
        bool finished = false;
        std::string state_path;
        std::unique_ptr<Run> run;
    };

    Server(Engine &eng, size_t hbm_budget_bytes, int max_live);
    ~Server();
    // Queue a solve of `steps` RK steps that arrived at `arrival` (seconds on clock()).
    int64_t submit(const LaserSlabParams &p, int precision, int64_t steps, double arrival,
                   const std::string &state_path, int poisson = kPoissonLU);
    // Admit what fits, advance every live solve one step, retire the finished ones.
    // Returns the number of solves still live.
    int step(double now);
    const Request &request(int64_t id) const;
    double clock() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
    }
    size_t used_bytes() const { return used_; }
    int live() const { return (int)live_.size(); }
    int waiting() const { return (int)waiting_.size(); }
    static size_t estimate_bytes(const LaserSlabParams &p, int precision);

private:
    void admit(double now);
    Engine &eng;
    size_t budget_, used_ = 0;
    int max_live_;
    int64_t next_id_ = 1;
    std::map<int64_t, Request> reqs_;
    std::deque<int64_t> waiting_;
    std::vector<int64_t> live_;
    std::vector<int64_t> finished_order_;
    std::chrono::steady_clock::time_point t0_ = std::chrono::steady_clock::now();
};

}  // namespace vx
