// C++ host interface over the C ABI, with the names and argument meanings of the
// reference's driver-facing class (SolverManager, SolverManager.hpp:5-19):
//   CalculateDt(cfl), Advance(dt), AdvanceFields(dt), reGrid(t)
// Errors become exceptions (the reference calls exit).  Header only; link against
// veritas_gb300/libvx_cuda.so.
#pragma once
#include <stdexcept>
#include <string>
#include <vector>

#include "vx.h"

namespace veritas_gb300 {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
    if (rc != VX_OK) throw Error(rc, vx_last_error());
}

// One GPU and one CUDA stream.
class Context {
public:
    explicit Context(int device = 0) { check(vx_ctx_create(device, &ctx_)); }
    ~Context() {
        if (ctx_) vx_ctx_destroy(ctx_);
    }
    Context(const Context &) = delete;
    Context &operator=(const Context &) = delete;
    vx_ctx *get() const { return ctx_; }
    void sync() const { check(vx_ctx_sync(ctx_)); }

private:
    vx_ctx *ctx_ = nullptr;
};

// SolverManager (SolverManager.hpp:5-19): Settings, one mesh per species and the field
// solver of one solve, resident on the context's GPU.
class SolverManager {
public:
    SolverManager(Context &ctx, const vx_problem &problem) { check(vx_run_create(ctx.get(), &problem, &run_)); }
    ~SolverManager() {
        if (run_) vx_run_destroy(run_);
    }
    SolverManager(const SolverManager &) = delete;
    SolverManager &operator=(const SolverManager &) = delete;

    // SolverManager::CalculateDt (SolverManager.cpp:162-164).  The CFL number comes from
    // the problem (Settings::cfl), which is what the reference's driver passes.
    double CalculateDt(double /*cfl*/ = 0.0) {
        double dt = 0.0;
        check(vx_run_calculate_dt(run_, &dt));
        return dt;
    }
    // SolverManager::Advance (SolverManager.cpp:28-39)
    void Advance(double timeStep) { check(vx_run_advance(run_, timeStep)); }
    // SolverManager::AdvanceFields (SolverManager.cpp:41-46)
    void AdvanceFields(double timeStep) { check(vx_run_advance_fields(run_, timeStep)); }
    // SolverManager::reGrid (SolverManager.cpp:48-57); t is only printed by the reference
    void reGrid(double /*t*/ = 0.0) { check(vx_run_regrid(run_)); }

    double time() const {
        double t = 0.0;
        check(vx_run_time(run_, &t));
        return t;
    }
    long long cells() const {
        int64_t c = 0;
        check(vx_run_cell_count(run_, &c));
        return (long long)c;
    }
    void saveState(const std::string &path) const { check(vx_run_save_state(run_, path.c_str())); }
    void loadState(const std::string &path) { check(vx_run_load_state(run_, path.c_str())); }
    vx_run *get() const { return run_; }

private:
    vx_run *run_ = nullptr;
};

}  // namespace veritas_gb300
