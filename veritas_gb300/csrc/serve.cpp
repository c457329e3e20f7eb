// Serving loop: continuous batching of independent solves on one context.
//
// Requests queue in arrival order.  Each call of step() advances every live solve by one
// full RK step in one batched launch set per precision (one launch per sub-step for all
// of them).  While that step runs on the GPU, the loop binds the runs the worker threads
// have finished, admits, in order, the waiting requests whose device-memory estimate fits
// in what the budget has left and hands them to the workers, which construct each run
// (host quadrature, clustering, Poisson factors, uploads) on their own engines and
// streams, and builds the launch sets of the next step's mix; the estimate is replaced by
// the run's real footprint when it is bound.  After the step each solve regrids by the reference driver's rule (veritas.cpp:146-151: a
// counter of steps since the last regrid; at a count above 20, once the plasma is on,
// SolverManager::reGrid and the counter restarts) — on a worker thread, the solve out of
// the batch until its new hierarchy is in place.  A solve whose CFL bound or
// E_x0 is not finite after its step (something in it went non-finite) fails and is
// retired alone; the others in the batch are unaffected (runs share launches, never data).  Finished solves
// write their final state where the request asked and release their memory before the
// next admission.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "serve.hpp"

namespace vx {

size_t Run::device_bytes() const {
    size_t b = 0;
    for (auto &sp : rects)
        for (auto &lvl : sp)
            for (auto &r : lvl) b += r->slab.bytes + r->cols.bytes + r->masks.bytes;
    for (const DevBuf *d : {&dBy, &dBz, &dEy, &dEz, &dAy, &dAz, &dasq, &dphi, &dcharge, &dJ, &dneut, &defin, &dex0,
                            &dasq32, &defin32, &dacell32, &drelc32, &dlu_perm, &dlb_band, &dlb_fptr, &dlb_fcol, &dlb_fval, &dlb_slot,
                            &dlb_sload, &dlb_take, &dub_band, &dub_diag, &dub_rdiag, &dub_rdlo, &dub_fptr, &dub_fcol,
                            &dub_fval, &dpf_Y, &drelc, &drefc, &dghost_ops, &diface_ops, &dcsync_ops})
        b += d->bytes;
    return b;
}

// Device bytes a request will take: the base level's patch planes times a refinement
// allowance (each further level may cover the base once more at most in cells), plus
// the field arrays and the Poisson operator.
size_t Server::estimate_bytes(const LaserSlabParams &p, int precision) {
    const double levels = std::max(1u, p.Lfinest);
    const double cells = (double)(p.nx + 4) * (p.np / 8 * 8 + 8 + 4);
    const double esize = precision == kF32 ? 4.0 : 8.0;
    const double planes = precision == kF32 ? 23.0 : 28.0;  // FP32: no gamma / face planes
    const double nfine = p.nx * std::pow((double)p.r, levels - 1);
    const double fields = nfine * (8.0 * 6 + 16) * 8.0 + nfine * 24.0 * (precision == kF32 ? 1.0 : 2.0);
    return (size_t)(cells * planes * esize * levels + fields);
}

Server::Server(Engine &e, size_t budget, int max_live) : eng(e), budget_(budget), max_live_(max_live) {
    for (int w = 0; w < kWorkers; w++) {
        worker_eng_.emplace_back(new Engine(e.device));
        worker_eng_.back()->arena_cache_limit = (size_t)256 << 20;  // single-run sets only
    }
    VX_CUDA(cudaSetDevice(e.device));  // the worker engines' constructors made it current too
    for (int w = 0; w < kWorkers; w++) workers_.emplace_back([this, w] { worker_loop(worker_eng_[w].get()); });
}

Server::~Server() {
    {
        std::lock_guard<std::mutex> lk(mu_);
        stop_ = true;
    }
    cv_.notify_all();
    for (auto &t : workers_)
        if (t.joinable()) t.join();
    // runs still queued for a regrid point at the loop's engine; finished ones were handed
    // back to it: all go before the worker engines
    todo_.clear();
    built_.clear();
    for (auto &kv : reqs_) kv.second.run.reset();
    if (std::getenv("VX_TRACE_SERVE"))
        std::fprintf(stderr,
                     "vx serve loop [s]: idle bind %.3f, dt + launch %.3f, bind + admit %.3f, next sets %.3f, "
                     "step wait %.3f, retire + regrid hand-off %.3f; next mix predicted %d, missed %d\n",
                     phase_s_[0], phase_s_[1], phase_s_[2], phase_s_[3], phase_s_[4], phase_s_[5], hits_, misses_);
}

void Server::worker_loop(Engine *weng) {
    cudaSetDevice(weng->device);
    for (;;) {
        Build b;
        {
            std::unique_lock<std::mutex> lk(mu_);
            cv_.wait(lk, [&] { return stop_ || !todo_.empty(); });
            if (stop_) return;
            b = std::move(todo_.front());
            todo_.pop_front();
        }
        try {
            if (b.regrid) {
                // the loop synchronised the solve's last step and dropped its launch sets:
                // SolverManager::reGrid on this thread's streams while the batch steps on
                b.run->adopt(*weng);
                b.run->regrid(false);
                weng->sync();
            } else {
                b.run.reset(new Run(*weng, std::make_shared<LaserSlab>(b.params), b.precision));
                b.run->poisson = b.poisson;
                b.run->fast64 = b.fast64;
                b.run->init();
            }
            b.run->migrate(eng);  // drops this engine's sets; the loop's engine runs it from now on
        } catch (const std::exception &e) {
            cudaStreamSynchronize(weng->stream);
            if (b.regrid) b.run->migrate(eng);  // the loop retires it as failed
            else b.run.reset();
            b.error = e.what();
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            built_.push_back(std::move(b));
        }
        built_cv_.notify_all();
    }
}

int64_t Server::submit(const LaserSlabParams &p, int precision, int64_t steps, double arrival,
                       const std::string &state_path, int poisson, int regrid, int fast64) {
    if (steps <= 0) throw std::invalid_argument("a request needs at least one step");
    if (precision != kF64 && precision != kF32) throw std::invalid_argument("precision must be 64 or 32");
    if (poisson != kPoissonLU && poisson != kPoissonScan) throw std::invalid_argument("poisson must be 0 or 1");
    Request r;
    r.id = next_id_++;
    r.params = p;
    r.precision = precision;
    r.poisson = precision == kF32 ? kPoissonScan : poisson;
    r.regrid = regrid ? 1 : 0;
    r.fast64 = precision == kF64 ? (fast64 ? 1 : 0) : 0;
    r.steps = steps;
    r.arrival = arrival;
    r.state_path = state_path;
    r.estimate = estimate_bytes(p, precision);
    if (r.estimate > budget_)
        throw std::invalid_argument("request of about " + std::to_string(r.estimate >> 20) +
                                    " MiB is larger than the whole memory budget");
    waiting_.push_back(r.id);
    reqs_.emplace(r.id, std::move(r));
    return next_id_ - 1;
}

int Server::waiting() const { return (int)waiting_.size() + building_; }

void Server::admit(double now, int bound_meanwhile) {
    std::vector<Build> go;
    while (!waiting_.empty() &&
           (int)live_.size() + bound_meanwhile + regridding_ + building_ + (int)go.size() < max_live_) {
        Request &r = reqs_.at(waiting_.front());
        if (used_ + r.estimate > budget_) break;  // in order: the head blocks the queue
        waiting_.pop_front();
        r.admitted = now;
        r.status = kBuilding;
        used_ += r.estimate;
        Build b;
        b.id = r.id;
        b.params = r.params;
        b.precision = r.precision;
        b.poisson = r.poisson;
        b.fast64 = r.fast64;
        go.push_back(std::move(b));
    }
    if (go.empty()) return;
    building_ += (int)go.size();
    {
        std::lock_guard<std::mutex> lk(mu_);
        for (auto &b : go) todo_.push_back(std::move(b));
    }
    cv_.notify_one();
}

void Server::bind_built(double now, std::vector<int64_t> &into) {
    std::vector<Build> done;
    {
        std::lock_guard<std::mutex> lk(mu_);
        done.swap(built_);
    }
    if (done.empty()) return;
    for (auto &b : done) {
        Request &r = reqs_.at(b.id);
        if (b.regrid) {
            regridding_--;
            r.out = false;
            const size_t bytes = b.run->device_bytes();
            used_ += bytes - r.bytes;
            r.bytes = bytes;
            if (r.status == kCancelled) {  // withdrawn while regridding
                used_ -= r.bytes;
                continue;
            }
            r.run = std::move(b.run);
            if (!b.error.empty()) {
                r.error = "regrid failed: " + b.error;
                retire(r, kFailed, clock());
                continue;
            }
            r.regrids++;
            into.push_back(r.id);
            continue;
        }
        building_--;
        used_ -= r.estimate;
        if (r.status == kCancelled) continue;  // withdrawn while building: the run goes
        if (!b.run) {
            r.error = b.error;
            r.status = kFailed;
            r.finish = clock();
            finished_order_.push_back(r.id);
            continue;
        }
        r.run = std::move(b.run);
        r.bytes = r.run->device_bytes();
        used_ += r.bytes;
        r.bound = now;
        r.status = kLive;
        into.push_back(r.id);
    }
    std::sort(into.begin(), into.end());  // arrival order, whatever came back when
}

void Server::retire(Request &r, Status st, double now) {
    r.finish = now;
    r.status = st;
    if (r.run) {
        r.sim_time = r.run->S->time;
        if (st == kDone && !r.state_path.empty()) r.run->save_state(r.state_path);
        r.cells = r.run->cell_count();
        used_ -= r.bytes;
        r.run.reset();
    }
    finished_order_.push_back(r.id);
}

void Server::cancel(int64_t id) {
    auto it = reqs_.find(id);
    if (it == reqs_.end()) throw std::invalid_argument("unknown request id");
    Request &r = it->second;
    switch (r.status) {
        case kWaiting:
            waiting_.erase(std::find(waiting_.begin(), waiting_.end(), id));
            r.status = kCancelled;
            r.finish = clock();
            finished_order_.push_back(id);
            break;
        case kBuilding:
            r.status = kCancelled;  // bind_built drops the run when its build ends
            r.finish = clock();
            break;
        case kLive:
            if (r.out) {  // bind_built drops the run when its regrid ends
                r.status = kCancelled;
                r.finish = clock();
                finished_order_.push_back(id);
                break;
            }
            eng.sync();
            live_.erase(std::find(live_.begin(), live_.end(), id));
            retire(r, kCancelled, clock());
            break;
        default:
            break;  // already over
    }
}

// One launch set per precision, Poisson solver and FP64 kernel form (different kernels).
static std::vector<std::vector<Run *>> partition(const std::vector<Run *> &set) {
    std::vector<std::vector<Run *>> parts;
    for (int prec : {kF64, kF32})
        for (int pois : {kPoissonLU, kPoissonScan})
            for (int fast : {0, 1}) {
                std::vector<Run *> part;
                for (Run *r : set)
                    if (r->precision == prec && r->poisson == pois && r->fast64 == fast) part.push_back(r);
                if (!part.empty()) parts.push_back(part);
            }
    return parts;
}

bool Server::regrid_due(const Request &r, double t_before) const {
    // the reference driver's rule, with the time before the step (veritas.cpp:146-151)
    return r.regrid && regrid_enabled && r.run->S->maxDepth > 0 && r.regrid_counter > 20 && t_before > regrid_after;
}

int Server::step(double now) {
    // VX_TRACE_SERVE=1: wall time of the loop's phases, summed over steps, on stderr at the end
    static const bool trace = std::getenv("VX_TRACE_SERVE") != nullptr;
    double tp = clock();
    auto phase = [&](int k) {
        if (!trace) return;
        const double t = clock();
        phase_s_[k] += t - tp;
        tp = t;
    };
    if (live_.empty()) {  // otherwise the previous step bound and admitted while it ran
        bind_built(now, live_);
        admit(now);
        if (live_.empty() && building_ + regridding_ > 0) {
            // nothing to step: wait (a little) for a build or a regrid to end rather than spin
            {
                std::unique_lock<std::mutex> lk(mu_);
                built_cv_.wait_for(lk, std::chrono::milliseconds(50), [&] { return !built_.empty(); });
            }
            bind_built(clock(), live_);
        }
        phase(0);
        if (live_.empty()) return regridding_;
    }
    if (trace) (live_ == predicted_ ? hits_ : misses_)++;
    std::vector<Run *> set;
    for (int64_t id : live_) set.push_back(reqs_.at(id).run.get());
    std::vector<std::vector<Run *>> used = partition(set);
    std::map<Run *, double> t_before, dt_of;
    for (Run *r : set) t_before[r] = r->S->time;
    for (auto &part : used) {
        auto dt = eng.calculate_dt(part);
        for (size_t k = 0; k < part.size(); k++) dt_of[part[k]] = dt[k];
        eng.advance(part, dt);
    }
    phase(1);
    // While the step runs: bind what the workers finished, admit, and build the host
    // tables of the launch sets of the next step's mix as far as it is known now — the
    // solves that neither finish nor regrid after this step, and the runs just bound.  A
    // solve that fails or is cancelled meanwhile changes the mix; its sets are then built
    // at the next step as before.
    std::vector<int64_t> fresh;
    bind_built(clock(), fresh);
    admit(clock(), (int)fresh.size());
    std::vector<Run *> next;
    {
        std::vector<int64_t> ids;
        for (int64_t id : live_) {
            const Request &r = reqs_.at(id);
            if (r.done_steps + 1 < r.steps && !regrid_due(r, t_before[r.run.get()])) ids.push_back(id);
        }
        ids.insert(ids.end(), fresh.begin(), fresh.end());
        std::sort(ids.begin(), ids.end());
        for (int64_t id : ids) next.push_back(reqs_.at(id).run.get());
        if (trace) predicted_ = ids;
    }
    phase(2);
    auto next_parts = partition(next);
    for (auto &part : next_parts) eng.prepare(part);
    phase(3);
    // the sets of earlier mixes are dropped, so cached tables do not pile up beside the budget
    std::vector<std::vector<Run *>> keep = used;
    keep.insert(keep.end(), next_parts.begin(), next_parts.end());
    eng.retain_sets(keep);
    // health: E_x0 (updated every stage from phi, which the solve makes depend on every
    // cell's charge) turns non-finite within a step once any f, charge or field value has
    // gone non-finite
    std::vector<double> ex0(set.size(), 0.0);
    for (size_t k = 0; k < set.size(); k++)
        VX_CUDA(cudaMemcpyAsync(&ex0[k], set[k]->F.ex0, sizeof(double), cudaMemcpyDeviceToHost, eng.stream));
    eng.sync();
    eng.flush_prepared();  // the next sets' table copies, queued now that the stream is idle
    phase(4);
    std::map<Run *, double> ex0_of;
    for (size_t k = 0; k < set.size(); k++) ex0_of[set[k]] = ex0[k];
    const double tnow = clock();
    std::vector<int64_t> still;
    std::vector<Build> regrids;
    for (int64_t id : live_) {
        Request &r = reqs_.at(id);
        Run *run = r.run.get();
        // health: the step's CFL bound (from the fields it started from) and E_x0 after it
        const double dt = dt_of[run];
        if (!(std::isfinite(dt) && dt > 0) || !std::isfinite(ex0_of[run])) {
            r.error = "the solve is not finite any more (CFL bound or E_x0 after step " +
                      std::to_string(r.done_steps + 1) + ")";
            retire(r, kFailed, tnow);
            continue;
        }
        r.done_steps++;
        if (r.done_steps >= r.steps) {
            retire(r, kDone, tnow);
            continue;
        }
        // The regrid runs on a worker thread while the others step on; the solve sits out
        // of the batch until it is back, so its own sequence (step, regrid, step) and bits
        // are those of a plain run.
        if (regrid_due(r, t_before[run])) {
            r.regrid_counter = 0;
            eng.forget(run);  // the step is synchronised above
            Build b;
            b.id = id;
            b.regrid = true;
            b.run = std::move(r.run);
            r.out = true;
            regridding_++;
            regrids.push_back(std::move(b));
            continue;
        }
        if (r.regrid && regrid_enabled && run->S->maxDepth > 0) r.regrid_counter++;
        still.push_back(id);
    }
    still.insert(still.end(), fresh.begin(), fresh.end());
    std::sort(still.begin(), still.end());  // arrival order
    live_ = still;
    if (!regrids.empty()) {
        {
            std::lock_guard<std::mutex> lk(mu_);
            for (auto it = regrids.rbegin(); it != regrids.rend(); ++it) todo_.push_front(std::move(*it));
        }
        cv_.notify_all();
    }
    phase(5);
    return (int)live_.size() + regridding_;
}

const Server::Request &Server::request(int64_t id) const {
    auto it = reqs_.find(id);
    if (it == reqs_.end()) throw std::invalid_argument("unknown request id");
    return it->second;
}

}  // namespace vx
